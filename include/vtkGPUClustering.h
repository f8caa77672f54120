/*
 * vtkGPUClustering.h -- reference-side binding of the GB300 clustering engine.
 *
 * Header-only C++ for a build of ACVD (valette/ACVD): include it after the
 * reference's own headers.  It replaces the energy minimisation of the
 * clustering engine, the virtual vtkUniformClustering<Metric>::MinimizeEnergy()
 * (Common/vtkUniformClustering.h:264,725-830), with the GPU engine behind the C
 * ABI of acvd_gpu.h.  Everything around it -- SetInput, SetNumberOfClusters,
 * SetSubsamplingThreshold, the curvature pre-processing, InitSamples, Remesh,
 * BuildDelaunayTriangulation, GetOutput -- stays the reference's own code.
 *
 *   typedef vtkGPUMetric<vtkQEMetricForClustering> GPUQEMetric;
 *   typedef vtkGPUClustering<vtkVerticesProcessing<vtkDiscreteRemeshing<GPUQEMetric> >, GPUQEMetric>
 *       vtkGPUQIsotropicDiscreteRemeshing;
 *   vtkGPUQIsotropicDiscreteRemeshing* r = vtkGPUQIsotropicDiscreteRemeshing::New();
 *   r->SetInput(mesh); r->SetNumberOfClusters(20000); r->GetMetric()->SetGradation(1.5);
 *   r->SetUnconstrainedInitialization(1); r->Remesh(); vtkSurface* out = r->GetOutput();
 *
 * vtkGPUMetric<M> is the reference metric M plus a copy of the curvature data
 * handed to it (SetCurvatureInfo, vtkDiscreteRemeshing.h:783) -- the metric keeps
 * them private, and the anisotropic metric overwrites its principal-direction
 * array in BuildMetric.  The engine's only extra state is the device ordinal and
 * whether a minimisation already ran: vtkDiscreteRemeshing's ForceManifold loop
 * re-enters MinimizeEnergy with IsClusterFreezed set, which is forwarded, as are
 * FixedClusters and the QEM clusters' AnchorItem (ACVDQ's fixed vertices).
 * Errors of the C ABI are thrown as std::runtime_error; there is no CPU fallback.
 */
#ifndef VTK_GPU_CLUSTERING_H
#define VTK_GPU_CLUSTERING_H

#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "acvd_gpu.h"

// whether a metric's Cluster has the QEM metric's AnchorItem member
template <class C, class = void>
struct acvd_has_anchor : std::false_type {};
template <class C>
struct acvd_has_anchor<C, decltype((void)std::declval<C&>().AnchorItem)> : std::true_type {};

template <class M>
struct acvd_metric_of {
    enum { value = -1 };
};
#ifdef _VTKISOTROPICMETRICFORCLUSTERING_H_
template <>
struct acvd_metric_of<vtkIsotropicMetricForClustering> {
    enum { value = ACVD_METRIC_ISOTROPIC };
};
#endif
#ifdef _VTKQEMETRICFORCLUSTERING_H_
template <>
struct acvd_metric_of<vtkQEMetricForClustering> {
    enum { value = ACVD_METRIC_QEM };
};
#endif
#ifdef _VTKQUADRICANISOTROPICMETRICFORCLUSTERING_H_
template <>
struct acvd_metric_of<vtkQuadricAnisotropicMetricForClustering> {
    enum { value = ACVD_METRIC_QUADRIC_ANISOTROPIC };
};
#endif

// The reference metric plugin, plus a copy of its curvature inputs and options.
template <class M>
class vtkGPUMetric : public M {
public:
    enum { acvd_metric = acvd_metric_of<M>::value };

    void SetCurvatureInfo(vtkDataArrayCollection* info) {
        vtkDoubleArray* ind = (vtkDoubleArray*)info->GetItem(0);
        Indicator.resize(ind->GetNumberOfTuples());
        for (vtkIdType i = 0; i < (vtkIdType)Indicator.size(); i++) Indicator[i] = ind->GetValue(i);
        PrincipalDirections.clear();
        if (info->GetNumberOfItems() > 1) {
            vtkFloatArray* pd = (vtkFloatArray*)info->GetItem(1);
            const vtkIdType n = pd->GetNumberOfTuples() * pd->GetNumberOfComponents();
            PrincipalDirections.resize(n);
            for (vtkIdType i = 0; i < n; i++) PrincipalDirections[i] = pd->GetValue(i);
        }
        M::SetCurvatureInfo(info);
    }

    void SetQuadricsOptimizationLevel(int level) {
        Level = level;
        M::SetQuadricsOptimizationLevel(level);
    }

    std::vector<double> Indicator;
    std::vector<float> PrincipalDirections;
    int Level = 3;
};

// Remesher: a reference vertex-clustering class instantiated on vtkGPUMetric<M>,
// e.g. vtkVerticesProcessing<vtkDiscreteRemeshing<vtkGPUMetric<M> > >.
template <class Remesher, class GPUMetric>
class vtkGPUClustering : public Remesher {
public:
    static vtkGPUClustering* New() { return new vtkGPUClustering; }

    void SetDevice(int d) { this->Device = d; }
    const acvd_stats& GetLastStats() const { return this->LastStats; }

protected:
    vtkGPUClustering() {}
    ~vtkGPUClustering() {}

    int Device = 0;
    bool Minimized = false;
    acvd_stats LastStats = {};

    void collect_anchors(std::vector<int32_t>& out, bool& any, std::true_type) {
        out.resize(this->NumberOfClusters);
        for (int c = 0; c < this->NumberOfClusters; c++) {
            out[c] = (int32_t)this->GetCluster(c)->AnchorItem;
            any = any || out[c] >= 0;
        }
    }
    void collect_anchors(std::vector<int32_t>&, bool&, std::false_type) {}

    static void check(acvd_ctx* ctx, int code, const char* what) {
        if (code == ACVD_OK) return;
        std::string msg = std::string(what) + ": " + (ctx ? acvd_last_error(ctx) : "no context");
        if (ctx) acvd_destroy(ctx);
        throw std::runtime_error(msg);
    }

    // MinimizeEnergy() on the GPU: the mesh, the metric inputs and the current
    // clustering (after FillHoles-free InitSamples) go to the device; the converged
    // clustering comes back and the reference's own ReComputeStatistics() rebuilds
    // its cluster records for BuildDelaunayTriangulation.
    void MinimizeEnergy() override {
        vtkSurface* mesh = this->GetInput();
        const vtkIdType nv = mesh->GetNumberOfPoints();
        const vtkIdType nf = mesh->GetNumberOfCells();
        const vtkIdType ne = mesh->GetNumberOfEdges();
        std::vector<double> xyz(3 * nv);
        for (vtkIdType i = 0; i < nv; i++) mesh->GetPointCoordinates(i, &xyz[3 * i]);
        std::vector<int32_t> tri(3 * nf), row(nv + 1), col, ev(2 * ne);
        for (vtkIdType f = 0; f < nf; f++) {
            vtkIdType a, b, c;
            mesh->GetFaceVertices(f, a, b, c);
            tri[3 * f] = (int32_t)a; tri[3 * f + 1] = (int32_t)b; tri[3 * f + 2] = (int32_t)c;
        }
        for (vtkIdType e = 0; e < ne; e++) {
            vtkIdType a, b;
            mesh->GetEdgeVertices(e, a, b);
            ev[2 * e] = (int32_t)a; ev[2 * e + 1] = (int32_t)b;
        }
        col.reserve(2 * ne);
        for (vtkIdType v = 0; v < nv; v++) {
            row[v] = (int32_t)col.size();
            vtkIdType n, *edges;
            mesh->GetVertexNeighbourEdges(v, n, edges);
            for (vtkIdType j = 0; j < n; j++) {
                vtkIdType a, b;
                mesh->GetEdgeVertices(edges[j], a, b);
                col.push_back((int32_t)(a == v ? b : a));
            }
        }
        row[nv] = (int32_t)col.size();

        acvd_opts opts;
        acvd_default_opts(&opts);
        opts.device = this->Device;
        opts.max_loops = this->MaxNumberOfLoops;
        opts.max_convergences = this->MaxNumberOfConvergences;
        acvd_ctx* ctx = acvd_create(&opts);
        if (!ctx) throw std::runtime_error("acvd_create: no usable CUDA device");
        GPUMetric& metric = this->MetricContext;
        const int id = GPUMetric::acvd_metric;
        const double g = metric.GetGradation();
        const bool use_ind = id == ACVD_METRIC_QUADRIC_ANISOTROPIC ? g != 0.0 : g > 0.0;
        check(ctx, acvd_set_mesh(ctx, nv, xyz.data(), nf, tri.data(), row.data(), col.data(), ne, ev.data()),
              "acvd_set_mesh");
        check(ctx, acvd_set_metric(ctx, id, use_ind ? metric.Indicator.data() : nullptr,
                                   metric.PrincipalDirections.empty() ? nullptr : metric.PrincipalDirections.data(),
                                   g),
              "acvd_set_metric");
        check(ctx, acvd_set_quadrics_optimization_level(ctx, metric.Level), "acvd_set_quadrics_optimization_level");
        // a re-entry (vtkDiscreteRemeshing's ForceManifold loop) finds the metric
        // already switched to constrained placement
        check(ctx, acvd_set_unconstrained_initialization(ctx, this->UnconstrainedInitialization && !this->Minimized),
              "acvd_set_unconstrained_initialization");
        check(ctx, acvd_set_labels(ctx, this->NumberOfClusters, this->Clustering->GetPointer(0)), "acvd_set_labels");
        // IsClusterFreezed (vtkUniformClustering.h:329), set by DetectNonManifoldOutputVertices
        std::vector<uint8_t> frozen(this->NumberOfClusters, 0);
        bool any_frozen = false;
        for (int c = 0; c < this->NumberOfClusters; c++) {
            frozen[c] = this->IsClusterFreezed->GetValue(c) ? 1 : 0;
            any_frozen = any_frozen || frozen[c];
        }
        if (any_frozen) check(ctx, acvd_set_frozen_clusters(ctx, frozen.data()), "acvd_set_frozen_clusters");
        // FixedClusters (vtkUniformClustering.h:134) and, for the QEM metric, every
        // cluster's AnchorItem (vtkQEMetricForClustering.h:127-128)
        if (this->FixedClusters && this->FixedClusters->GetNumberOfIds() > 0) {
            std::vector<int32_t> f(this->FixedClusters->GetNumberOfIds());
            for (size_t i = 0; i < f.size(); i++) f[i] = (int32_t)this->FixedClusters->GetId((vtkIdType)i);
            check(ctx, acvd_set_fixed_clusters(ctx, (int32_t)f.size(), f.data()), "acvd_set_fixed_clusters");
        }
        std::vector<int32_t> anchors;
        bool any_anchor = false;
        collect_anchors(anchors, any_anchor, acvd_has_anchor<typename GPUMetric::Cluster>());
        if (any_anchor)
            check(ctx, acvd_set_anchor_items(ctx, (int32_t)anchors.size(), anchors.data()), "acvd_set_anchor_items");
        check(ctx, acvd_minimize(ctx, &this->LastStats), "acvd_minimize");
        check(ctx, acvd_get_labels(ctx, this->Clustering->GetPointer(0)), "acvd_get_labels");
        acvd_destroy(ctx);
        this->NumberOfLoops += this->LastStats.sweeps;
        // the state the reference's own loop ends in (:778-790)
        if (this->UnconstrainedInitialization) this->MetricContext.SetConstrainedClustering(1);
        this->ConnexityConstraint = 1;
        this->Minimized = true;
        this->ReComputeStatistics();
    }
};

#endif  // VTK_GPU_CLUSTERING_H

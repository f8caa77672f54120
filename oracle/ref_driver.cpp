// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own clustering code -- Common/vtkUniformClustering.h,
// DiscreteRemeshing/vtkSurfaceClustering.h, DiscreteRemeshing/vtkVerticesProcessing.h
// and the three metric headers, compiled unmodified from the reference tree
// against oracle/shim (see oracle/Makefile) -- behind the same C ABI as the C++
// restatement in acvd_port.cpp (prefix ref_ instead of port_).  The build exists
// only where the reference sources are present; its outputs pin the restatement
// (tests/test_oracle_pin.py) and generate tests/golden/.
#include "vtkSurfaceClustering.h"
#include "vtkVerticesProcessing.h"
#include "vtkIsotropicMetricForClustering.h"
#include "vtkQEMetricForClustering.h"
#include "vtkQuadricAnisotropicMetricForClustering.h"
#include "vtkCurvatureMeasure.h"

#include <chrono>
#include <type_traits>

// Exposes the protected members of the reference engine; nothing is overridden.
template <class M>
class Probe : public vtkVerticesProcessing<vtkSurfaceClustering<M>> {
public:
    typedef vtkVerticesProcessing<vtkSurfaceClustering<M>> Base;
    Probe() {}
    using Base::Init;
    using Base::InitSamples;
    using Base::MinimizeEnergy;
    using Base::ReComputeStatistics;
    using Base::ComputeGlobalEnergy;
    using Base::CleanClustering;
    using Base::FillHolesInClustering;
    using Base::Clusters;
    using Base::Clustering;
    using Base::ClustersSizes;
    using Base::ConnexityConstraint;
    using Base::NumberOfLoops;
    using Base::UnconstrainedInitialization;
    using Base::MetricContext;
};

struct RefBase {
    virtual ~RefBase() {}
    virtual void set_option(const char* name, double v) = 0;
    virtual void init(const int* initial) = 0;
    virtual double run() = 0;
    virtual double process(const int* initial) = 0;
    virtual void get_labels(int* out) = 0;
    virtual void evaluate(const int* lab, int constrained) = 0;
    virtual double global_energy() = 0;
    virtual void get_clusters(double* S, double* W, double* Q, double* C, double* E, int* sz) = 0;
    virtual int clean() = 0;
    virtual int fill() = 0;
    virtual void set_labels(const int* lab) = 0;
    virtual int loops() = 0;
    virtual void post_placement(int level, double* out) = 0;
    virtual void curvature(double* indicator, float* principal_dirs) = 0;
    virtual void set_fixed(int n, const int* ids) = 0;
    virtual int set_anchors(int n, const int* anchors) = 0;
};

template <class M>
struct Ref : RefBase {
    Probe<M>* p = nullptr;
    vtkIdList* fixed = nullptr;   // the engine keeps the pointer (SetFixedClusters)
    long long n = 0;
    int K = 0;

    Ref(long long nV, const double* pts, long long nF, const int* tri,
        const double* indicator, const float* pdirs, double gradation, int k) {
        n = nV; K = k;
        vtkSurface* mesh = vtkSurface::New();
        mesh->CreateFromArrays(nV, pts, nF, tri);
        p = new Probe<M>;
        p->SetInput(mesh);
        mesh->Delete();
        p->SetNumberOfClusters(k);
        p->SetConsoleOutput(0);
        p->SetDisplay(0);
        p->GetMetric()->SetGradation(gradation);
        if (indicator) {
            vtkDataArrayCollection* coll = vtkDataArrayCollection::New();
            vtkDoubleArray* ind = vtkDoubleArray::New();
            ind->SetNumberOfValues(nV);
            for (long long i = 0; i < nV; i++) ind->SetValue(i, indicator[i]);
            coll->AddItem(ind);
            ind->Delete();
            if (pdirs) {
                vtkFloatArray* pd = vtkFloatArray::New();
                pd->SetNumberOfValues(6 * nV);
                for (long long i = 0; i < 6 * nV; i++) pd->SetValue(i, pdirs[i]);
                coll->AddItem(pd);
                pd->Delete();
            }
            p->GetMetric()->SetCurvatureInfo(coll);
            coll->Delete();
        }
    }
    ~Ref() override {
        p->Delete();
        if (fixed) fixed->Delete();
    }

    // what ACVDQ.cxx:327-334 does with a list of fixed vertices
    void set_fixed(int nf, const int* ids) override {
        if (fixed) fixed->Delete();
        fixed = vtkIdList::New();
        for (int i = 0; i < nf; i++) fixed->InsertNextId(ids[i]);
        p->SetFixedClusters(fixed);
    }
    int set_anchors(int na, const int* anchors) override {
        if constexpr (std::is_same<M, vtkQEMetricForClustering>::value) {
            for (int c = 0; c < na; c++) p->GetCluster(c)->AnchorItem = anchors[c];
            return 0;
        }
        return -1;
    }

    void set_option(const char* name, double v) override {
        if (!std::strcmp(name, "unconstrained_init")) p->SetUnconstrainedInitialization((int)v);
        else if (!std::strcmp(name, "max_loops")) p->SetMaxNumberOfLoops((int)v);
        else if (!std::strcmp(name, "max_convergences")) p->SetMaxNumberOfConvergences((int)v);
        else if (!std::strcmp(name, "connexity")) p->ConnexityConstraint = (int)v;
#ifdef DOmultithread
        else if (!std::strcmp(name, "threads")) p->SetNumberOfThreads((int)v);
        else if (!std::strcmp(name, "pooling_ratio")) p->SetPoolingRatio((int)v);
#endif
        else if (!std::strcmp(name, "constrained")) p->GetMetric()->SetConstrainedClustering((int)v);
        else if (!std::strcmp(name, "level")) {
            if constexpr (!std::is_same<M, vtkIsotropicMetricForClustering>::value)
                p->GetMetric()->SetQuadricsOptimizationLevel((int)v);
        }
    }
    void set_initial(const int* initial) {
        vtkIntArray* a = vtkIntArray::New();
        a->SetNumberOfValues(n);
        for (long long i = 0; i < n; i++) a->SetValue(i, initial[i]);
        p->SetInitialClustering(a);
        a->Delete();
    }
    void init(const int* initial) override {
        if (initial) set_initial(initial);
        p->Init();
        p->InitSamples(0);
    }
    double run() override {
        auto t0 = std::chrono::steady_clock::now();
        if (p->UnconstrainedInitialization) p->MetricContext.SetConstrainedClustering(0);
        p->MinimizeEnergy();
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    double process(const int* initial) override {
        if (initial) set_initial(initial);
        auto t0 = std::chrono::steady_clock::now();
        p->ProcessClustering();
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void get_labels(int* out) override { for (long long i = 0; i < n; i++) out[i] = p->Clustering->GetValue(i); }
    void set_labels(const int* lab) override { for (long long i = 0; i < n; i++) p->Clustering->SetValue(i, lab[i]); }
    void evaluate(const int* lab, int constrained) override {
        p->Init();
        p->GetMetric()->SetConstrainedClustering(constrained);
        set_labels(lab);
        p->ReComputeStatistics();
    }
    double global_energy() override { return (double)p->ComputeGlobalEnergy(); }
    void get_clusters(double* S, double* W, double* Q, double* C, double* E, int* sz) override {
        for (int k = 0; k < K; k++) {
            auto* c = p->GetCluster(k);
            for (int j = 0; j < 3; j++) S[3 * k + j] = c->SValue[j];
            W[k] = c->SWeight;
            if constexpr (std::is_same<M, vtkIsotropicMetricForClustering>::value) {
                for (int j = 0; j < 9; j++) Q[9 * k + j] = 0;
            } else {
                for (int j = 0; j < 9; j++) Q[9 * k + j] = c->SQuadric[j];
            }
            p->GetMetric()->GetClusterCentroid(c, C + 3 * k);
            E[k] = p->GetMetric()->GetClusterEnergy(c);
            sz[k] = p->GetClusterSize(k);
        }
    }
    int clean() override { return p->CleanClustering(); }
    int fill() override {
        p->FillHolesInClustering(p->Clustering);
        int bad = 0;
        for (long long i = 0; i < n; i++) { const int c = p->Clustering->GetValue(i); if (c < 0 || c >= K) bad++; }
        return bad;
    }
    int loops() override { return p->NumberOfLoops; }
    // The post-placement loop of DiscreteRemeshing/Examples/ACVD.cxx:217-291 (a driver
    // program, restated here as a loop) over the reference's own
    // vtkQuadricTools::AddTriangleQuadric / ComputeRepresentativePoint and the
    // metric's GetClusterCentroid (the output vertices of BuildDelaunayTriangulation,
    // vtkDiscreteRemeshing.h:1024-1033).  Needs the cluster statistics (evaluate).
    // What vtkDiscreteRemeshing::SamplingPreProcessing runs for vertex clustering
    // (DiscreteRemeshing/vtkDiscreteRemeshing.h:630-637): the reference's own
    // vtkCurvatureMeasure, polynomial fitting (method 1) on vertices with its
    // default 3-ring neighbourhood and principal directions on.
    void curvature(double* indicator, float* principal_dirs) override {
        vtkCurvatureMeasure* cm = vtkCurvatureMeasure::New();
        cm->SetInputData(p->GetInput());
        cm->SetComputationMethod(1);
        cm->SetElementsType(1);
        cm->SetComputePrincipalDirections(1);
        vtkDataArrayCollection* coll = cm->GetCurvatureIndicator();
        vtkDoubleArray* ind = (vtkDoubleArray*)coll->GetItem(0);
        vtkFloatArray* pd = (vtkFloatArray*)coll->GetItem(1);
        for (long long i = 0; i < n; i++) indicator[i] = ind->GetValue(i);
        for (long long i = 0; i < 6 * n; i++) principal_dirs[i] = pd->GetValue(i);
        cm->Delete();
    }
    void post_placement(int level, double* out) override {
        vtkSurface* mesh = p->GetInput();
        std::vector<double> Q(9 * (size_t)K, 0.0);
        vtkIdList* fl = vtkIdList::New();
        for (long long i = 0; i < n; i++) {
            const int c = p->Clustering->GetValue(i);
            if (c < 0 || c >= K) continue;
            mesh->GetVertexNeighbourFaces(i, fl);
            for (vtkIdType j = 0; j < fl->GetNumberOfIds(); j++)
                vtkQuadricTools::AddTriangleQuadric(&Q[9 * (size_t)c], mesh, fl->GetId(j), false);
        }
        fl->Delete();
        int valid = 0;
        for (int k = 0; k < K; k++) if (p->ClustersSizes->GetValue(k) > 0) { valid = k; break; }
        for (int k = 0; k < K; k++) {
            double P[3];
            p->GetMetric()->GetClusterCentroid(p->GetCluster(p->ClustersSizes->GetValue(k) == 0 ? valid : k), P);
            vtkQuadricTools::ComputeRepresentativePoint(&Q[9 * (size_t)k], P, level);
            out[3 * k] = P[0]; out[3 * k + 1] = P[1]; out[3 * k + 2] = P[2];
        }
    }
};

// Built twice: as is (prefix ref_, the sequential engine) and with DOmultithread,
// the reference's own switch that makes vtkSurfaceClustering derive from
// vtkThreadedClustering (ACVDQP), plus ACVD_REF_THREADED for the prefix refmt_.
#ifdef ACVD_REF_THREADED
#define REF_FN(x) refmt_##x
#else
#define REF_FN(x) ref_##x
#endif

extern "C" {

void* REF_FN(create)(int metric, long long nV, const double* pts, long long nF, const int* tri,
                 const double* indicator, const float* pdirs, double gradation, int K) {
    if (metric == 0) return new Ref<vtkIsotropicMetricForClustering>(nV, pts, nF, tri, indicator, pdirs, gradation, K);
    if (metric == 1) return new Ref<vtkQEMetricForClustering>(nV, pts, nF, tri, indicator, pdirs, gradation, K);
    return new Ref<vtkQuadricAnisotropicMetricForClustering>(nV, pts, nF, tri, indicator, pdirs, gradation, K);
}
void REF_FN(destroy)(void* h) { delete (RefBase*)h; }
int REF_FN(set_option)(void* h, const char* name, double v) { ((RefBase*)h)->set_option(name, v); return 0; }
void REF_FN(init)(void* h, const int* initial) { ((RefBase*)h)->init(initial); }
double REF_FN(run)(void* h) { return ((RefBase*)h)->run(); }
double REF_FN(process)(void* h, const int* initial) { return ((RefBase*)h)->process(initial); }
void REF_FN(get_labels)(void* h, int* out) { ((RefBase*)h)->get_labels(out); }
void REF_FN(set_labels)(void* h, const int* lab) { ((RefBase*)h)->set_labels(lab); }
void REF_FN(evaluate)(void* h, const int* lab, int constrained) { ((RefBase*)h)->evaluate(lab, constrained); }
double REF_FN(global_energy)(void* h) { return ((RefBase*)h)->global_energy(); }
void REF_FN(get_clusters)(void* h, double* S, double* W, double* Q, double* C, double* E, int* sz) {
    ((RefBase*)h)->get_clusters(S, W, Q, C, E, sz);
}
int REF_FN(clean)(void* h) { return ((RefBase*)h)->clean(); }
int REF_FN(fill_holes)(void* h) { return ((RefBase*)h)->fill(); }
int REF_FN(loops)(void* h) { return ((RefBase*)h)->loops(); }
void REF_FN(post_placement)(void* h, int level, double* out) { ((RefBase*)h)->post_placement(level, out); }
void REF_FN(set_fixed)(void* h, int n, const int* ids) { ((RefBase*)h)->set_fixed(n, ids); }
int REF_FN(set_anchors)(void* h, int n, const int* anchors) { return ((RefBase*)h)->set_anchors(n, anchors); }
void REF_FN(curvature)(void* h, double* indicator, float* principal_dirs) {
    ((RefBase*)h)->curvature(indicator, principal_dirs);
}

}  // extern "C"

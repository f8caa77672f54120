// ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product library.
//
// CPU restatement of ACVD's discrete Voronoi clustering path (sequential, FP64),
// written from the behaviour of the reference files cited at each function:
//   engine    Common/vtkUniformClustering.h            (MinimizeEnergy, ProcessOneLoop, ...)
//   adapter   DiscreteRemeshing/vtkVerticesProcessing.h (items = vertices, edges = mesh edges)
//   metrics   DiscreteRemeshing/vtkIsotropicMetricForClustering.h,
//             DiscreteRemeshing/vtkQEMetricForClustering.h,
//             DiscreteRemeshing/vtkQuadricAnisotropicMetricForClustering.h
//   quadrics  Common/vtkQuadricTools.cxx
//   mesh      Common/vtkSurfaceBase.cxx (edge table, vertex rings), Common/vtkSurface.cxx (areas)
//   dual mesh DiscreteRemeshing/vtkDiscreteRemeshing.h:956-1152
// The arithmetic follows the reference expression by expression so that, given the
// same VTK math (oracle/restated_math.h), its results match the reference's own
// headers compiled against oracle/shim bit for bit (tests/test_oracle_pin.py).
// It is the checker for the CUDA path and the CPU baseline timed by bench.py.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <queue>
#include <thread>
#include <random>
#include <type_traits>
#include <vector>

#include "restated_math.h"
#include "port_mesh.h"

namespace port {

// vtkQuadricTools::ComputeDisplacement (.cxx:83-163), threshold 1e-3 (.h:36)
static int compute_displacement(const double* Q, const double* p, double* disp, int maxUsed,
                                double thr = 0.001) {
    double A[3][3], U[3][3], VT[3][3], b[3], w[3], T[3][3], T2[3][3];
    int rank_def = 0;
    b[0] = -Q[3]; b[1] = -Q[6]; b[2] = -Q[8];
    A[0][0] = Q[0]; A[0][1] = A[1][0] = Q[1]; A[0][2] = A[2][0] = Q[2];
    A[1][1] = Q[4]; A[1][2] = A[2][1] = Q[5]; A[2][2] = Q[7];
    rmath::svd3(A, U, w, VT);
    double absw[3], maxW = -1.0;
    for (int j = 0; j < 3; j++) { absw[j] = std::fabs(w[j]); if (absw[j] > maxW) maxW = absw[j]; }
    const double invmaxW = 1.0 / maxW;
    for (int i = 0; i < 3; i++) {
        double lmax = -1; int im = -1;
        for (int j = 0; j < 3; j++) if (lmax < absw[j]) { lmax = absw[j]; im = j; }
        if ((absw[im] * invmaxW > thr) && (maxUsed > 0)) {
            const double inv = 1.0 / w[im];
            T[im][0] = U[0][im] * inv; T[im][1] = U[1][im] * inv; T[im][2] = U[2][im] * inv;
        } else {
            T[im][0] = T[im][1] = T[im][2] = 0; rank_def++;
        }
        absw[im] = -2; maxUsed--;
    }
    rmath::transpose33(VT, VT);
    rmath::mul33(VT, T, T2);
    rmath::mul33v(A, p, disp);
    for (int i = 0; i < 3; i++) disp[i] = b[i] - disp[i];
    rmath::mul33v(T2, disp, disp);
    return rank_def;
}

// vtkQuadricTools::ComputeRepresentativePoint (.cxx:168-177)
static int representative_point(const double* Q, double* p, int maxUsed) {
    double d[3];
    const int r = compute_displacement(Q, p, d, maxUsed);
    for (int i = 0; i < 3; i++) p[i] += d[i];
    return r;
}

// ClampWeights (vtkIsotropicMetricForClustering.h:273-291 and siblings)
template <class ItemT>
static void clamp_weights(std::vector<ItemT>& it, double ratio) {
    double avg = 0;
    for (auto& x : it) avg += x.w;
    avg /= (double)it.size();
    const double mn = avg / ratio, mx = avg * ratio;
    for (auto& x : it) { if (x.w > mx) x.w = mx; if (x.w < mn) x.w = mn; }
}

// ---------------------------------------------------------------------------
// Metrics (the plugin concept of the reference: Item, Cluster, Add/Sub,
// ComputeClusterCentroid, ComputeClusterEnergy)
// ---------------------------------------------------------------------------
struct IsoMetric {   // vtkIsotropicMetricForClustering.h
    struct Item { double v[3]; double w; };
    struct Cluster { double S[3]; double W; double E; };
    std::vector<Item> items;
    const Mesh* mesh = nullptr;
    double gradation = 0; const double* indicator = nullptr;
    void set_constrained(int) {}
    void reset(Cluster* c) const { c->S[0] = c->S[1] = c->S[2] = 0; c->W = 0; c->E = 0; }
    double weight(idt i) const { return items[i].w; }
    void add(idt i, Cluster* c) const {
        const Item& I = items[i];
        c->S[0] += I.v[0]; c->S[1] += I.v[1]; c->S[2] += I.v[2]; c->W += I.w;
    }
    void sub(idt i, Cluster* c) const {
        const Item& I = items[i];
        c->S[0] -= I.v[0]; c->S[1] -= I.v[1]; c->S[2] -= I.v[2]; c->W -= I.w;
    }
    void centroid(Cluster*) const {}
    void energy(Cluster* c) const {
        c->E = (-c->S[0] * c->S[0] - c->S[1] * c->S[1] - c->S[2] * c->S[2]) / c->W;
    }
    void get_centroid(const Cluster* c, double* p) const {
        p[0] = c->S[0] / c->W; p[1] = c->S[1] / c->W; p[2] = c->S[2] / c->W;
    }
    void build(const Mesh& m) {   // BuildMetric, vertex items (:244-266)
        mesh = &m;
        items.resize(m.nV);
        for (idt i = 0; i < m.nV; i++) {
            const double a = m.vertex_area(i);
            items[i].w = indicator ? a * std::pow(indicator[i], gradation) : a;
            m.point(i, items[i].v);
        }
        clamp_weights(items, 100000);
        for (auto& I : items) { I.v[0] *= I.w; I.v[1] *= I.w; I.v[2] *= I.w; }
    }
    void accum(const Cluster* c, double* S, double* W, double* Q) const {
        for (int k = 0; k < 3; k++) S[k] = c->S[k];
        *W = c->W;
        for (int k = 0; k < 9; k++) Q[k] = 0;
    }
};

struct QEMMetric {   // vtkQEMetricForClustering.h
    struct Item { double Q[9]; double v[3]; double w; };
    struct Cluster {
        double E; double SQ[9]; double c[3]; double S[3]; double W; char rank; idt anchor;
        Cluster() : E(0), W(0), rank(0), anchor(-1) {
            for (double& x : SQ) x = 0; for (double& x : c) x = 0; for (double& x : S) x = 0;
        }
    };
    std::vector<Item> items;
    const Mesh* mesh = nullptr;
    double gradation = 0; const double* indicator = nullptr;
    int active = 1, level = 3;
    void set_constrained(int c) { active = c; }
    void reset(Cluster* c) const {
        for (double& x : c->SQ) x = 0; for (double& x : c->S) x = 0; for (double& x : c->c) x = 0;
        c->W = 0; c->E = 0;
    }
    double weight(idt i) const { return items[i].w; }
    void add(idt i, Cluster* c) const {
        const Item& I = items[i];
        for (int k = 0; k < 3; k++) c->S[k] += I.v[k];
        for (int k = 0; k < 9; k++) c->SQ[k] += I.Q[k];
        c->W += I.w;
    }
    void sub(idt i, Cluster* c) const {
        const Item& I = items[i];
        for (int k = 0; k < 3; k++) c->S[k] -= I.v[k];
        for (int k = 0; k < 9; k++) c->SQ[k] -= I.Q[k];
        c->W -= I.w;
        if (c->anchor == i) c->anchor = -2;
    }
    void centroid(Cluster* c) const {   // :268-285
        if (c->anchor >= 0) { mesh->point(c->anchor, c->c); return; }
        for (int k = 0; k < 3; k++) c->c[k] = c->S[k] / c->W;
        if (!active || !level) return;
        c->rank = (char)representative_point(c->SQ, c->c, level);
    }
    void energy(Cluster* c) const {     // :194-208
        if (c->anchor == -2) { c->E = 1e100; return; }
        c->E = (c->c[0] * c->c[0] + c->c[1] * c->c[1] + c->c[2] * c->c[2]) * c->W
               - 2.0 * (c->c[0] * c->S[0] + c->c[1] * c->S[1] + c->c[2] * c->S[2]);
    }
    void get_centroid(const Cluster* c, double* p) const { for (int k = 0; k < 3; k++) p[k] = c->c[k]; }
    void build(const Mesh& m) {   // BuildMetric, vertex items (:325-342)
        mesh = &m;
        items.resize(m.nV);
        for (idt i = 0; i < m.nV; i++) {
            items[i].w = m.vertex_area(i);
            if (gradation > 0) items[i].w *= std::pow(indicator[i], gradation);
        }
        clamp_weights(items, 10000);
        std::vector<idt> fl;
        for (idt i = 0; i < m.nV; i++) {   // ComputeVertexQuadric (:151-167)
            Item& I = items[i];
            const double w = I.w;
            for (double& x : I.Q) x = 0;
            m.vertex_faces(i, fl);
            for (idt f : fl) m.add_triangle_quadric(I.Q, f);
            m.point(i, I.v);
            for (int k = 0; k < 3; k++) I.v[k] = I.v[k] * w;
            I.w = w;
        }
    }
    void accum(const Cluster* c, double* S, double* W, double* Q) const {
        for (int k = 0; k < 3; k++) S[k] = c->S[k];
        *W = c->W;
        for (int k = 0; k < 9; k++) Q[k] = c->SQ[k];
    }
};

struct AnisoMetric {   // vtkQuadricAnisotropicMetricForClustering.h
    struct Item { float v[3]; float w; float T[6]; float TX[3]; double Q[9]; };
    struct Cluster {
        double S[3]; double W; double E; double ST[6]; double STX[3]; double c[3]; double SQ[9];
    };
    std::vector<Item> items;
    const Mesh* mesh = nullptr;
    double gradation = 0; const double* indicator = nullptr; const float* pdirs = nullptr;
    int level = 3;
    void set_constrained(int) {}   // :61, no-op
    void reset(Cluster* c) const { std::memset(c, 0, sizeof(Cluster)); }
    double weight(idt i) const { return items[i].w; }
    void add(idt i, Cluster* c) const {
        const Item& I = items[i];
        for (int k = 0; k < 3; k++) { c->S[k] += (double)I.v[k]; c->STX[k] += (double)I.TX[k]; }
        for (int k = 0; k < 6; k++) c->ST[k] += (double)I.T[k];
        for (int k = 0; k < 9; k++) c->SQ[k] += (double)I.Q[k];
        c->W += (double)I.w;
    }
    void sub(idt i, Cluster* c) const {
        const Item& I = items[i];
        for (int k = 0; k < 3; k++) { c->S[k] -= (double)I.v[k]; c->STX[k] -= (double)I.TX[k]; }
        for (int k = 0; k < 6; k++) c->ST[k] -= (double)I.T[k];
        for (int k = 0; k < 9; k++) c->SQ[k] -= (double)I.Q[k];
        c->W -= (double)I.w;
    }
    void centroid(Cluster* c) const {   // :282-288
        c->c[0] = c->S[0] / c->W; c->c[1] = c->S[1] / c->W; c->c[2] = c->S[2] / c->W;
        representative_point(c->SQ, c->c, level);
    }
    void energy(Cluster* c) const {     // :168-184
        const double x = c->c[0], y = c->c[1], z = c->c[2];
        const double* T = c->ST;
        c->E = T[0] * x * x + T[3] * y * y + T[5] * z * z
               + 2.0 * T[1] * x * y + 2.0 * T[2] * x * z + 2.0 * T[4] * y * z;
        const double* U = c->STX;
        c->E -= 2.0 * (x * U[0] + y * U[1] + z * U[2]);
    }
    void get_centroid(const Cluster* c, double* p) const { for (int k = 0; k < 3; k++) p[k] = c->c[k]; }
    void build(const Mesh& m) {   // BuildMetric, vertex items (:374-487)
        mesh = &m;
        items.resize(m.nV);
        std::vector<idt> fl;
        for (idt i = 0; i < m.nV; i++) {
            Item& I = items[i];
            for (double& x : I.Q) x = 0;                      // ComputeVertexQuadric (:524-539)
            m.vertex_faces(i, fl);
            for (idt f : fl) m.add_triangle_quadric(I.Q, f);
            if (gradation == 0) I.w = (float)m.vertex_area(i);
            else I.w = (float)(m.vertex_area(i) * std::pow(indicator[i], gradation));
            double p[3]; m.point(i, p);
            I.v[0] = (float)p[0]; I.v[1] = (float)p[1]; I.v[2] = (float)p[2];
        }
        {   // ClampWeights, ratio 1e5 (:401, :489-508)
            double avg = 0;
            for (auto& I : items) avg += I.w;
            avg = avg / (double)items.size();
            const double mn = avg / 100000, mx = avg * 100000;
            for (auto& I : items) {
                if (I.w > mx) I.w = (float)mx;
                if (I.w < mn) I.w = (float)mn;
            }
        }
        for (idt i = 0; i < m.nV; i++) {
            Item& I = items[i];
            const double area = m.vertex_area(i);
            double PD[6];
            for (int j = 0; j < 6; j++) PD[j] = (double)pdirs[i * 6 + j];
            // Area*(d1 d1^T + d2 d2^T) in compact form; entry 3 uses PD[5]^2 in place of
            // PD[4]^2 exactly as the reference does (:442-446)
            I.T[0] = (float)(area * PD[0] * PD[0] + area * PD[3] * PD[3]);
            I.T[1] = (float)(area * PD[0] * PD[1] + area * PD[3] * PD[4]);
            I.T[2] = (float)(area * PD[0] * PD[2] + area * PD[3] * PD[5]);
            I.T[3] = (float)(area * PD[1] * PD[1] + area * PD[5] * PD[5]);
            I.T[4] = (float)(area * PD[1] * PD[2] + area * PD[4] * PD[5]);
            I.T[5] = (float)(area * PD[2] * PD[2] + area * PD[5] * PD[5]);
            I.TX[0] = I.T[0] * I.v[0] + I.T[1] * I.v[1] + I.T[2] * I.v[2];
            I.TX[1] = I.T[1] * I.v[0] + I.T[3] * I.v[1] + I.T[4] * I.v[2];
            I.TX[2] = I.T[2] * I.v[0] + I.T[4] * I.v[1] + I.T[5] * I.v[2];
            I.v[0] *= I.w; I.v[1] *= I.w; I.v[2] *= I.w;
        }
    }
    void accum(const Cluster* c, double* S, double* W, double* Q) const {
        for (int k = 0; k < 3; k++) S[k] = c->S[k];
        *W = c->W;
        for (int k = 0; k < 9; k++) Q[k] = c->SQ[k];
    }
};

// ---------------------------------------------------------------------------
// Engine (Common/vtkUniformClustering.h) + vertex adapter (vtkVerticesProcessing.h)
// ---------------------------------------------------------------------------
struct EngineBase {
    virtual ~EngineBase() {}
    Mesh mesh;
    int K = 0;
    std::vector<int> labels;       // Clustering
    std::vector<int> initial;      // InitialClustering
    std::vector<int> sizes;        // ClustersSizes
    std::vector<int> last_mod;     // ClustersLastModification
    std::vector<unsigned char> frozen;
    std::vector<idt> fixed;        // FixedClusters (:134, :332): cluster c < fixed.size() holds item fixed[c]
    std::vector<unsigned char> edges_last_loop;
    unsigned char rel_loops = 1;
    int n_loops = 0;
    int connexity = 0;
    int unconstrained_init = 0;
    int sampling_type = 1;
    int max_convergences = 1000000000;
    int max_loops = 5000000;
    std::queue<idt> queue;

    // ACVDQP: the threaded engine vtkThreadedClustering (DiscreteRemeshing/
    // vtkThreadedClustering.h), selected by threads > 0 as DOmultithread selects it
    // (vtkSurfaceClustering.h:44-52).  The mesh is split into pool_size - 1 regions
    // (the engine's own random sampling, holes filled); an edge belongs to its region
    // when both ends lie in it, else to the serial process pool_size - 1.  Each loop,
    // `threads` threads take regions longest-first from a priority queue and run the
    // edge test under per-cluster locks; the main thread then runs the serial process.
    int threads = 0;              // SetNumberOfThreads; 0 = the sequential engine
    int pooling_ratio = 5;        // SetPoolingRatio (ctor :990-1012)
    int pool_size = 0;            // PoolingRatio * NumberOfThreads + 1 (Init :749)
    std::vector<int> edge_proc;   // EdgesProcess (ComputeEdgesLayout :806-888)
    // ProcessesQueues1/2 (:752-759): queue [owner * pool_size + pusher]; a process only
    // pushes into its own pusher column, so concurrent processes never share a queue
    std::vector<std::queue<idt>> queues_a, queues_b;
    std::vector<std::queue<idt>>* push_q = &queues_a;
    std::vector<std::queue<idt>>* pop_q = &queues_b;
    // vtkPriorityQueue as the reference uses it: the smallest priority pops first, an id
    // already queued is not inserted again
    struct RegionQueue {
        std::vector<std::pair<double, int>> h;
        void insert(double pr, int id) {
            for (const auto& x : h)
                if (x.second == id) return;
            h.push_back({pr, id});
            std::push_heap(h.begin(), h.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
        }
        int pop() {
            if (h.empty()) return -1;
            std::pop_heap(h.begin(), h.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
            const int id = h.back().second;
            h.pop_back();
            return id;
        }
    };
    RegionQueue pool_a, pool_b;
    RegionQueue* pool1 = &pool_a;      // PoolQueue1 / PoolQueue2, swapped after each loop
    RegionQueue* pool2 = &pool_b;
    std::mutex pool_lock1, pool_lock2;   // PoolAllocationLock, PoolAllocationLock2
    std::unique_ptr<std::mutex[]> cluster_locks;   // ClustersLocks (K + 1)
    int n_cluster_locks = 0;
    long long collisions = 0;          // NumberOfLockingCollisions (summed after a loop)

    // labels read and written concurrently by the threads (the reference's races on
    // Clustering, benign there), as relaxed atomics
    int lab_get(idt i) const { return __atomic_load_n(&labels[i], __ATOMIC_RELAXED); }
    void lab_set(idt i, int v) { __atomic_store_n(&labels[i], v, __ATOMIC_RELAXED); }

    // Init's part of vtkThreadedClustering (:746-772) with ComputeEdgesLayout type 1
    void threaded_init() {
        pool_size = pooling_ratio * threads + 1;
        std::vector<int> region(n_items());
        random_sampling(region, pool_size - 1);
        fill_holes_in(region);
        edge_proc.assign(mesh.n_edges(), 0);
        for (idt e = 0; e < mesh.n_edges(); e++) {
            int c1 = region[mesh.ev1[e]];
            if (c1 >= pool_size || c1 < 0) c1 = pool_size - 1;
            if (region[mesh.ev2[e]] != c1) c1 = pool_size - 1;
            edge_proc[e] = c1;
        }
        queues_a.assign((size_t)pool_size * pool_size, std::queue<idt>());
        queues_b.assign((size_t)pool_size * pool_size, std::queue<idt>());
        push_q = &queues_a;
        pop_q = &queues_b;
        pool_a.h.clear();
        pool_b.h.clear();
        pool1 = &pool_a;
        pool2 = &pool_b;
        collisions = 0;
    }

    // FillQueuesFromClustering of the threaded engine (:203-240)
    void threaded_fill_queue() {
        for (auto& q : *push_q)
            while (!q.empty()) q.pop();
        for (idt e = 0; e < mesh.n_edges(); e++)
            if (labels[mesh.ev1[e]] != labels[mesh.ev2[e]])
                (*push_q)[(size_t)edge_proc[e] * pool_size + edge_proc[e]].push(e);
        for (int i = 0; i < pool_size - 1; i++) pool1->insert(i, i);
    }

    // AddEdgeToProcess / AddItemRingToProcess of the threaded engine (:125-131, :108-114)
    void push_edge(idt e, int process) { (*push_q)[(size_t)edge_proc[e] * pool_size + process].push(e); }
    void push_ring(idt item, int process) { for (idt e : mesh.ring[item]) push_edge(e, process); }

    // ConnexityConstraintProblemLocal with the labels read as the threads see them
    int connexity_problem_threaded(idt item, int cluster) const {
        if (!connexity) return 0;
        std::vector<idt> vl;
        for (idt e : mesh.ring[item]) {
            const idt v1 = mesh.ev1[e], v2 = mesh.ev2[e];
            if (v1 != item && lab_get(v1) == cluster) vl.push_back(v1);
            if (v2 != item && lab_get(v2) == cluster) vl.push_back(v2);
        }
        return connected_set(vl);
    }

    // statistics of the last MinimizeEnergy
    int stat_convergences = 0;
    long long stat_moves = 0;
    double stat_seconds = 0;

    virtual void build_metric() = 0;
    virtual void set_constrained(int c) = 0;
    virtual void recompute_statistics() = 0;
    virtual int process_one_loop() = 0;
    virtual int threaded_loop() = 0;
    virtual double item_weight(idt i) const = 0;
    virtual double cluster_energy(int k) const = 0;
    virtual void cluster_accum(int k, double* S, double* W, double* Q, double* c) const = 0;
    // a new empty cluster (vtkDiscreteRemeshing.h:257-269)
    virtual void add_cluster() = 0;
    virtual void remove_last_cluster() = 0;
    // Cluster::AnchorItem of the QEM metric (vtkQEMetricForClustering.h:127-128);
    // false for the metrics without it
    virtual bool set_anchor(int, idt) { return false; }

    idt n_items() const { return mesh.nV; }

    // vtkVerticesProcessing::ConnexityConstraintProblemLocal (:168-237)
    int connexity_problem(idt item, int cluster) const {
        if (!connexity) return 0;
        std::vector<idt> vl;
        for (idt e : mesh.ring[item]) {
            const idt v1 = mesh.ev1[e], v2 = mesh.ev2[e];
            if (v1 != item && labels[v1] == cluster) vl.push_back(v1);
            if (v2 != item && labels[v2] == cluster) vl.push_back(v2);
        }
        return connected_set(vl);
    }

    // 0 when the vertices of vl are connected through mesh edges among themselves
    // (the BFS of ConnexityConstraintProblemLocal, vtkVerticesProcessing.h:199-235)
    int connected_set(std::vector<idt>& vl) const {
        if (vl.empty()) return 0;
        const size_t total = vl.size();
        size_t visited = 1;
        std::queue<idt> q;
        idt v = vl[0];
        vl.erase(vl.begin());
        q.push(v);
        while (!q.empty()) {
            const idt a = q.front(); q.pop();
            for (idt e : mesh.ring[a]) {
                const idt b = mesh.ev1[e], c = mesh.ev2[e];
                for (size_t j = 0; j < vl.size(); j++) {
                    if (vl[j] == b || vl[j] == c) {
                        q.push(vl[j]); visited++;
                        vl.erase(vl.begin() + j);
                        break;
                    }
                }
            }
        }
        return visited == total ? 0 : 1;
    }

    void add_ring_to_queue(idt item) { for (idt e : mesh.ring[item]) queue.push(e); }

    // ReComputeClustersSize (:353-373)
    void recompute_sizes() {
        std::fill(sizes.begin(), sizes.end(), 0);
        for (idt i = 0; i < n_items(); i++) {
            const int c = labels[i];
            if (c >= 0 && c < K) sizes[c]++;
        }
    }

    // CleanClustering (:406-549); returns the number of clusters that had several components
    int clean_clustering() {
        const idt n = n_items();
        std::vector<char> visited(n, 0);
        std::vector<std::vector<std::pair<idt, int>>> extra(K);
        std::vector<idt> first(K, 0);
        std::vector<int> first_size(K, 0);
        std::vector<idt> nb;
        std::queue<idt> q;
        for (idt i = 0; i < n; i++) {
            if (visited[i] || labels[i] == K) continue;
            while (!q.empty()) q.pop();
            int size = 0;
            q.push(i);
            const int type = labels[i];
            // the component holding the cluster's fixed item outweighs any other (:439-447)
            const idt fixed_item = type < (int)fixed.size() ? fixed[type] : -1;
            while (!q.empty()) {
                const idt a = q.front(); q.pop();
                if (visited[a]) continue;
                size += a == fixed_item ? 1000000000 : 1;
                visited[a] = 1;
                mesh.vertex_neighbours(a, nb);
                for (idt b : nb) if (!visited[b] && labels[b] == type) q.push(b);
            }
            if (first[type] == 0) { first[type] = i; first_size[type] = size; }
            else {
                if (extra[type].empty()) extra[type].push_back({first[type], first_size[type]});
                extra[type].push_back({i, size});
            }
        }
        std::fill(visited.begin(), visited.end(), 0);
        int number = 0;
        for (int k = 0; k < K; k++) {
            if (extra[k].empty()) continue;
            number++;
            int smax = 0, imax = 0;
            for (size_t j = 0; j < extra[k].size(); j++) {
                if (smax >= extra[k][j].second) continue;
                smax = extra[k][j].second; imax = (int)j;
            }
            for (size_t j = 0; j < extra[k].size(); j++) {
                if ((int)j == imax) continue;
                while (!q.empty()) q.pop();
                q.push(extra[k][j].first);
                const int type = labels[extra[k][j].first];
                while (!q.empty()) {
                    const idt a = q.front(); q.pop();
                    if (visited[a]) continue;
                    visited[a] = 1;
                    labels[a] = K;
                    mesh.vertex_neighbours(a, nb);
                    for (idt b : nb) if (labels[b] == type) q.push(b);
                }
            }
        }
        return number;
    }

    // FillHolesInClustering (:552-633); returns the number of items left unassigned
    int fill_holes() { return fill_holes_in(labels); }
    // the same on another array (the threaded engine's regions); the connectivity test
    // reads the engine's own labels, as the reference's does
    int fill_holes_in(std::vector<int>& labels) {
        std::queue<idt> q;
        for (idt e = 0; e < mesh.n_edges(); e++) {
            const idt i1 = mesh.ev1[e], i2 = mesh.ev2[e];
            const int c1 = labels[i1], c2 = labels[i2];
            const bool bad1 = (c1 < 0) || (c1 >= K), bad2 = (c2 < 0) || (c2 >= K);
            if (bad1 != bad2) q.push(e);
        }
        while (!q.empty()) {
            const idt e = q.front(); q.pop();
            idt i1 = mesh.ev1[e], i2 = mesh.ev2[e];
            int c1 = labels[i1], c2 = labels[i2];
            if (c1 == K) { std::swap(i1, i2); c1 = c2; c2 = K; }
            if (c1 != K && c2 == K && this->connexity_problem(i2, c2) == 0) {
                labels[i2] = c1;
                add_ring_to(q, i2);
            }
        }
        int problems = 0;
        for (idt i = 0; i < n_items(); i++) if (labels[i] < 0 || labels[i] >= K) problems++;
        return problems;
    }
    void add_ring_to(std::queue<idt>& q, idt item) { for (idt e : mesh.ring[item]) q.push(e); }

    // FillQueuesFromClustering (:636-652)
    void fill_queue() {
        while (!queue.empty()) queue.pop();
        for (idt e = 0; e < mesh.n_edges(); e++)
            if (labels[mesh.ev1[e]] != labels[mesh.ev2[e]]) queue.push(e);
        queue.push(-1);
    }

    void set_all_modified() { for (int k = 0; k < K; k++) last_mod[k] = n_loops; }

    // Init (:1363-1381) + Allocate (:1349-1360)
    void init() {
        sizes.assign(K, 0);
        labels.assign(n_items(), K);
        last_mod.assign(K, 0);
        edges_last_loop.assign(mesh.n_edges(), 0);
        frozen.assign(K, 0);
        build_metric();
        rel_loops = 1;
        n_loops = 0;
        while (!queue.empty()) queue.pop();
        if (threads > 0) threaded_init();
    }

    // ComputeInitialRandomSampling (:1178-1316): the fixed items take clusters
    // 0 .. F-1, the grown regions the labels above them
    void initial_random_sampling() { random_sampling(labels, K); }
    // the same into another array with n_regions regions (the threaded engine's thread
    // regions, vtkThreadedClustering.h:851-858); unassigned items keep the label K
    void random_sampling(std::vector<int>& labels, int n_regions) {
        const idt n = n_items();
        for (idt i = 0; i < n; i++) labels[i] = K;
        const int offset = (int)fixed.size();
        for (int o = 0; o < offset; o++) labels[fixed[o]] = o;
        std::vector<int> itm(n);
        idt remaining_items = n;
        int remaining_regions = n_regions - offset;
        for (idt i = 0; i < n; i++) itm[i] = (int)i;
        std::mt19937 rng;
        rng.seed(0);
        for (idt i = n - 1; i > 0; --i) std::swap(itm[i], itm[rng() % n]);
        double sw = 0;
        for (idt i = 0; i < n; i++) sw += item_weight(i);
        const double target = sw / (double)n_regions;
        idt first = 0;
        std::queue<int> q;
        std::vector<idt> nb;
        while (remaining_items > 0 && remaining_regions > 0) {
            bool found = false;
            int item = 0;
            while (!found && first < n) {
                item = itm[first];
                if (labels[item] == K) found = true; else first++;
            }
            // the reference continues here, which with fixed items (never counted off
            // remaining_items) can repeat forever once every item is taken
            if (!found) break;
            while (!q.empty()) q.pop();
            q.push(item);
            sw = 0;
            remaining_regions--;
            while (!q.empty()) {
                item = q.front(); q.pop();
                if (labels[item] != K) continue;
                labels[item] = remaining_regions + offset;
                sw += item_weight(item);
                remaining_items--;
                mesh.vertex_neighbours(item, nb);
                for (idt b : nb) q.push((int)b);
                if (sw > target) break;
            }
        }
        if (remaining_regions == 0) return;
        std::fill(sizes.begin(), sizes.end(), 0);
        for (idt i = 0; i < n; i++) {
            itm[i] = (int)i;
            if (labels[i] == K) continue;
            sizes[labels[i]]++;
        }
        for (idt i = n - 1; i > 0; --i) std::swap(itm[i], itm[rng() % n]);
        first = 0;
        while (remaining_regions) {
            idt item;
            while (true) {
                item = itm[first];
                first++;
                const int cl = labels[item];
                if (cl == K) break;
                if (sizes[cl] == 1) continue;
                labels[item] = remaining_regions + offset;
                sizes[cl]--;
                sizes[remaining_regions + offset]++;
                break;
            }
            remaining_regions--;
            labels[item] = remaining_regions + offset;
        }
    }

    // InitSamples (:1124-1175), types 1 and 2
    void init_samples() {
        for (idt i = 0; i < n_items(); i++) labels[i] = K;
        if (sampling_type == 2) {
            for (idt i = 0; i < n_items(); i++) labels[i] = initial[i];
        } else {
            initial_random_sampling();
        }
    }

    // MinimizeEnergy (:725-830)
    void minimize_energy() {
        auto t0 = std::chrono::steady_clock::now();
        fill_holes();
        if (threads > 0) threaded_fill_queue(); else fill_queue();
        recompute_statistics();
        set_all_modified();
        int convergences = 0;
        int early = 0;
        for (int k = 0; k < K; k++) if (!frozen[k]) early += sizes[k];
        stat_moves = 0;
        while (true) {
            if (threads > 0) std::swap(push_q, pop_q);   // SwapQueues (:742, :743-747)
            const int mods = threads > 0 ? threaded_loop() : process_one_loop();
            stat_moves += mods;
            n_loops++;
            if (rel_loops == 255) {
                std::fill(edges_last_loop.begin(), edges_last_loop.end(), 0);
                rel_loops = 1;
            } else rel_loops++;
            if (mods == 0 || n_loops > max_loops || (mods <= early / 1000 && convergences <= 1)) {
                if (unconstrained_init && convergences == 0) set_constrained(1);
                if (convergences >= 1) connexity = 1;
                convergences++;
                const int disconnected = clean_clustering();
                fill_holes();
                recompute_sizes();
                if (disconnected == 0 && mods == 0) break;
                if (n_loops >= max_loops) break;
                if (convergences >= max_convergences) break;
                recompute_statistics();
                if (threads > 0) threaded_fill_queue(); else fill_queue();
                set_all_modified();
            }
        }
        stat_convergences = convergences;
        stat_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // ProcessClustering (:655-714) from the point where Init and InitSamples are done
    void process_clustering() {
        if (unconstrained_init) set_constrained(0);
        minimize_energy();
    }

    // ComputeGlobalEnergy (:1319-1346), bins as in the reference
    long double global_energy() const {
        long double energy = 0;
        const int nb = (int)std::sqrt((double)K);
        std::vector<long double> bins(nb, 0.0L);
        int bin = 0, count = 0;
        for (int k = 0; k < K; k++) {
            bins[bin] += (long double)cluster_energy(k);
            count++;
            if (count == nb && bin < nb - 1) bin++;
        }
        for (int i = 0; i < nb; i++) energy += bins[i];
        return energy;
    }
};

template <class M>
struct Engine : EngineBase {
    M metric;
    std::vector<typename M::Cluster> clusters;

    void build_metric() override { metric.build(mesh); }
    void set_constrained(int c) override { metric.set_constrained(c); }
    double item_weight(idt i) const override { return metric.weight(i); }
    double cluster_energy(int k) const override { return clusters[k].E; }
    void cluster_accum(int k, double* S, double* W, double* Q, double* c) const override {
        metric.accum(&clusters[k], S, W, Q);
        metric.get_centroid(&clusters[k], c);
    }

    void add_cluster() override {
        clusters.emplace_back();
        metric.reset(&clusters.back());
        frozen.push_back(0);
        last_mod.push_back(n_loops);
        sizes.push_back(0);
        K++;
    }
    void remove_last_cluster() override {
        clusters.pop_back();
        frozen.pop_back();
        last_mod.pop_back();
        sizes.pop_back();
        K--;
    }

    bool set_anchor(int k, idt item) override {
        if constexpr (std::is_same<M, QEMMetric>::value) {
            if (k < 0 || k >= K) return false;
            clusters[k].anchor = item;
            return true;
        }
        return false;
    }

    void set_k(int k) {   // SetNumberOfClusters (:62-69)
        K = k;
        clusters.resize(k);
        for (auto& c : clusters) metric.reset(&c);
    }

    void recompute_statistics() override {   // (:376-403)
        recompute_sizes();
        for (auto& c : clusters) metric.reset(&c);
        for (idt i = 0; i < n_items(); i++) {
            const int c = labels[i];
            if (c >= 0 && c < K) metric.add(i, &clusters[c]);
        }
        for (auto& c : clusters) { metric.centroid(&c); metric.energy(&c); }
    }

    // ProcessOneLoop of the threaded engine (vtkThreadedClustering.h:663-693) with its
    // thread body MyMainForClustering (:245-283)
    int threaded_loop() override {
        if (n_cluster_locks != K + 1) {
            cluster_locks.reset(new std::mutex[K + 1]);
            n_cluster_locks = K + 1;
        }
        std::vector<int> mods(threads + 1, 0);
        std::vector<long long> coll(threads + 1, 0);
        std::vector<std::thread> th;
        for (int t = 0; t < threads; t++) {
            th.emplace_back([this, t, &mods, &coll] {
                while (true) {
                    int process;
                    {
                        std::lock_guard<std::mutex> g(pool_lock1);
                        process = pool1->pop();
                    }
                    if (process < 0) break;
                    const auto t0 = std::chrono::steady_clock::now();
                    execute_process(process, mods[t], coll[t]);
                    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                    std::lock_guard<std::mutex> g(pool_lock2);
                    pool2->insert(-dt, process);
                }
            });
        }
        for (auto& x : th) x.join();
        execute_process(pool_size - 1, mods[threads], coll[threads]);
        std::swap(pool1, pool2);
        int total = 0;
        for (int t = 0; t <= threads; t++) {
            total += mods[t];
            collisions += coll[t];
        }
        return total;
    }

    // ExecuteProcess (vtkThreadedClustering.h:285-493): the process's pop queues, the
    // sequential loop's edge test under the two clusters' locks
    void execute_process(int process, int& mods, long long& coll) {
        typename M::Cluster c21, c22, c31, c32;
        auto lock = [&](int c) {
            if (!cluster_locks[c].try_lock()) {
                coll++;
                cluster_locks[c].lock();
            }
        };
        for (int cq = 0; cq < pool_size; cq++) {
            std::queue<idt>& q = (*pop_q)[(size_t)process * pool_size + cq];
            while (!q.empty()) {
                const idt edge = q.front();
                q.pop();
                const idt i1 = mesh.ev1[edge], i2 = mesh.ev2[edge];
                if (edges_last_loop[edge] == rel_loops || i2 < 0) continue;
                edges_last_loop[edge] = rel_loops;
                const int v1 = lab_get(i1), v2 = lab_get(i2);
                if (v1 == v2) continue;
                if (v1 < v2) { lock(v1); lock(v2); } else { lock(v2); lock(v1); }
                if (v1 == K) {
                    // I1 unassigned: joins I2's cluster (no modification stamp here, :344-354)
                    typename M::Cluster* c2 = &clusters[v2];
                    metric.add(i1, c2); metric.centroid(c2); metric.energy(c2);
                    sizes[v2]++;
                    push_ring(i1, process);
                    lab_set(i1, v2);
                    mods++;
                } else if (v2 == K) {
                    typename M::Cluster* c1 = &clusters[v1];
                    metric.add(i2, c1); metric.centroid(c1); metric.energy(c1);
                    sizes[v1]++;
                    push_ring(i2, process);
                    lab_set(i2, v1);
                    mods++;
                } else {
                    int result = 1;
                    typename M::Cluster* c1 = &clusters[v1];
                    typename M::Cluster* c2 = &clusters[v2];
                    if ((last_mod[v1] >= n_loops - 1 || last_mod[v2] >= n_loops - 1) && !frozen[v1] && !frozen[v2]) {
                        double try1, try2, try3;
                        try1 = c1->E + c2->E;
                        if (sizes[v1] == 1 || connexity_problem_threaded(i1, v1) == 1) try2 = 100000000.0;
                        else {
                            c21 = *c1; c22 = *c2;
                            metric.sub(i1, &c21); metric.add(i1, &c22);
                            metric.centroid(&c21); metric.centroid(&c22);
                            metric.energy(&c21); metric.energy(&c22);
                            try2 = c21.E + c22.E;
                        }
                        if (sizes[v2] == 1 || connexity_problem_threaded(i2, v2) == 1) try3 = 1000000000.0;
                        else {
                            c31 = *c1; c32 = *c2;
                            metric.sub(i2, &c32); metric.add(i2, &c31);
                            metric.centroid(&c31); metric.centroid(&c32);
                            metric.energy(&c31); metric.energy(&c32);
                            try3 = c31.E + c32.E;
                        }
                        if (try1 <= try2 && try1 <= try3) result = 1;
                        else if (try2 < try1 && try2 < try3) result = 2;
                        else result = 3;
                    }
                    if (result == 1) {
                        push_edge(edge, process);
                    } else if (result == 2) {
                        lab_set(i1, v2);
                        sizes[v2]++; sizes[v1]--;
                        *c1 = c21; *c2 = c22;
                        push_ring(i1, process);
                        mods++;
                        last_mod[v1] = n_loops; last_mod[v2] = n_loops;
                    } else {
                        lab_set(i2, v1);
                        sizes[v1]++; sizes[v2]--;
                        *c1 = c31; *c2 = c32;
                        push_ring(i2, process);
                        mods++;
                        last_mod[v1] = n_loops; last_mod[v2] = n_loops;
                    }
                }
                cluster_locks[v1].unlock();
                cluster_locks[v2].unlock();
            }
        }
    }

    int process_one_loop() override {   // (:833-995)
        typename M::Cluster c21, c22, c31, c32;
        int mods = 0;
        while (true) {
            const idt edge = queue.front();
            queue.pop();
            if (edge == -1) { queue.push(-1); return mods; }
            const idt i1 = mesh.ev1[edge], i2 = mesh.ev2[edge];
            if (edges_last_loop[edge] == rel_loops || i2 < 0) continue;
            edges_last_loop[edge] = rel_loops;
            const int v1 = labels[i1], v2 = labels[i2];
            if (v1 == v2) continue;
            if (v1 == K) {
                typename M::Cluster* c2 = &clusters[v2];
                metric.add(i1, c2); metric.centroid(c2); metric.energy(c2);
                sizes[v2]++;
                add_ring_to_queue(i1);
                mods++;
                labels[i1] = v2;
                last_mod[v2] = n_loops;
                continue;
            } else if (v2 == K) {
                typename M::Cluster* c1 = &clusters[v1];
                metric.add(i2, c1); metric.centroid(c1); metric.energy(c1);
                sizes[v1]++;
                add_ring_to_queue(i2);
                mods++;
                labels[i2] = v1;
                last_mod[v1] = n_loops;
                continue;
            }
            if ((last_mod[v1] < n_loops - 1 && last_mod[v2] < n_loops - 1) || frozen[v1] || frozen[v2]) {
                queue.push(edge);
                continue;
            }
            typename M::Cluster* c1 = &clusters[v1];
            typename M::Cluster* c2 = &clusters[v2];
            double try1, try2, try3;
            try1 = c1->E + c2->E;
            if (sizes[v1] == 1 || connexity_problem(i1, v1) == 1) try2 = 100000000.0;
            else {
                c21 = *c1; metric.sub(i1, &c21);
                c22 = *c2; metric.add(i1, &c22);
                metric.centroid(&c21); metric.centroid(&c22);
                metric.energy(&c21); metric.energy(&c22);
                try2 = c21.E + c22.E;
            }
            if (sizes[v2] == 1 || connexity_problem(i2, v2) == 1) try3 = 1000000000.0;
            else {
                c32 = *c2; metric.sub(i2, &c32);
                c31 = *c1; metric.add(i2, &c31);
                metric.centroid(&c31); metric.centroid(&c32);
                metric.energy(&c31); metric.energy(&c32);
                try3 = c31.E + c32.E;
            }
            if (try1 <= try2 && try1 <= try3) {
                queue.push(edge);
            } else if (try2 < try1 && try2 < try3) {
                labels[i1] = v2;
                sizes[v2]++; sizes[v1]--;
                *c1 = c21; *c2 = c22;
                add_ring_to_queue(i1);
                mods++;
                last_mod[v1] = n_loops; last_mod[v2] = n_loops;
            } else {
                labels[i2] = v1;
                sizes[v1]++; sizes[v2]--;
                *c1 = c31; *c2 = c32;
                add_ring_to_queue(i2);
                mods++;
                last_mod[v1] = n_loops; last_mod[v2] = n_loops;
            }
        }
    }
};

}  // namespace port

// ---------------------------------------------------------------------------
// C ABI for the tests and the CPU baseline (ctypes)
// ---------------------------------------------------------------------------
using namespace port;

struct PortHandle {
    EngineBase* eng = nullptr;
    int metric = 0;
    std::vector<double> indicator;
    std::vector<float> pdirs;
};

extern "C" {

// metric: 0 isotropic, 1 QEM, 2 quadric-anisotropic.  indicator/pdirs may be null.
void* port_create(int metric, long long nV, const double* pts, long long nF, const int* tri,
                  const double* indicator, const float* pdirs, double gradation, int K) {
    PortHandle* h = new PortHandle;
    h->metric = metric;
    if (indicator) h->indicator.assign(indicator, indicator + nV);
    if (pdirs) h->pdirs.assign(pdirs, pdirs + 6 * nV);
    EngineBase* e = nullptr;
    if (metric == 0) {
        auto* x = new Engine<IsoMetric>;
        x->metric.gradation = gradation;
        x->metric.indicator = indicator ? h->indicator.data() : nullptr;
        e = x; x->mesh.build(nV, pts, nF, tri); x->set_k(K);
    } else if (metric == 1) {
        auto* x = new Engine<QEMMetric>;
        x->metric.gradation = gradation;
        x->metric.indicator = indicator ? h->indicator.data() : nullptr;
        e = x; x->mesh.build(nV, pts, nF, tri); x->set_k(K);
    } else {
        auto* x = new Engine<AnisoMetric>;
        x->metric.gradation = gradation;
        x->metric.indicator = indicator ? h->indicator.data() : nullptr;
        x->metric.pdirs = h->pdirs.data();
        e = x; x->mesh.build(nV, pts, nF, tri); x->set_k(K);
    }
    h->eng = e;
    return h;
}

void port_destroy(void* hp) {
    PortHandle* h = (PortHandle*)hp;
    delete h->eng;
    delete h;
}

// name in {"level", "unconstrained_init", "max_loops", "max_convergences", "connexity"}
int port_set_option(void* hp, const char* name, double value) {
    PortHandle* h = (PortHandle*)hp;
    EngineBase* e = h->eng;
    if (!std::strcmp(name, "unconstrained_init")) e->unconstrained_init = (int)value;
    else if (!std::strcmp(name, "max_loops")) e->max_loops = (int)value;
    else if (!std::strcmp(name, "max_convergences")) e->max_convergences = (int)value;
    else if (!std::strcmp(name, "connexity")) e->connexity = (int)value;
    else if (!std::strcmp(name, "threads")) h->eng->threads = (int)value;
    else if (!std::strcmp(name, "pooling_ratio")) h->eng->pooling_ratio = (int)value;
    else if (!std::strcmp(name, "level")) {
        if (h->metric == 1) static_cast<Engine<QEMMetric>*>(e)->metric.level = (int)value;
        else if (h->metric == 2) static_cast<Engine<AnisoMetric>*>(e)->metric.level = (int)value;
    } else if (!std::strcmp(name, "constrained")) e->set_constrained((int)value);
    else return -1;
    return 0;
}

// Init + InitSamples.  initial may be null (random sampling, type 1) or N labels (type 2).
void port_init(void* hp, const int* initial) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    e->init();
    if (initial) { e->sampling_type = 2; e->initial.assign(initial, initial + e->n_items()); }
    else e->sampling_type = 1;
    e->init_samples();
}

// The remainder of ProcessClustering: unconstrained switch + MinimizeEnergy.
double port_run(void* hp) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    e->process_clustering();
    return e->stat_seconds;
}

void port_get_labels(void* hp, int* out) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    std::memcpy(out, e->labels.data(), sizeof(int) * e->n_items());
}

void port_set_labels(void* hp, const int* in) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    std::memcpy(e->labels.data(), in, sizeof(int) * e->n_items());
}

// Init() then load the labels and ReComputeStatistics -- the reference's own load path
// (vtkDiscreteRemeshing.h:915-932).  constrained sets the metric's placement switch.
void port_evaluate(void* hp, const int* lab, int constrained) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    e->init();
    e->set_constrained(constrained);
    std::memcpy(e->labels.data(), lab, sizeof(int) * e->n_items());
    e->recompute_statistics();
}

void port_recompute(void* hp) { ((PortHandle*)hp)->eng->recompute_statistics(); }

double port_global_energy(void* hp) { return (double)((PortHandle*)hp)->eng->global_energy(); }

// Per-cluster S (3K), W (K), Q (9K; zeros for the isotropic metric), centroid (3K),
// energy (K) and size (K).
void port_get_clusters(void* hp, double* S, double* W, double* Q, double* C, double* E, int* sizes) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    for (int k = 0; k < e->K; k++) {
        e->cluster_accum(k, S + 3 * k, W + k, Q + 9 * k, C + 3 * k);
        E[k] = e->cluster_energy(k);
        sizes[k] = e->sizes[k];
    }
}

// Items as the metric stores them: value (3, weight-multiplied), weight, quadric (9).
void port_get_items(void* hp, double* V, double* W, double* Q) {
    PortHandle* h = (PortHandle*)hp;
    EngineBase* e = h->eng;
    for (idt i = 0; i < e->n_items(); i++) {
        if (h->metric == 0) {
            auto& I = static_cast<Engine<IsoMetric>*>(e)->metric.items[i];
            for (int k = 0; k < 3; k++) V[3 * i + k] = I.v[k];
            W[i] = I.w;
            for (int k = 0; k < 9; k++) Q[9 * i + k] = 0;
        } else if (h->metric == 1) {
            auto& I = static_cast<Engine<QEMMetric>*>(e)->metric.items[i];
            for (int k = 0; k < 3; k++) V[3 * i + k] = I.v[k];
            W[i] = I.w;
            for (int k = 0; k < 9; k++) Q[9 * i + k] = I.Q[k];
        } else {
            auto& I = static_cast<Engine<AnisoMetric>*>(e)->metric.items[i];
            for (int k = 0; k < 3; k++) V[3 * i + k] = I.v[k];
            W[i] = I.w;
            for (int k = 0; k < 9; k++) Q[9 * i + k] = I.Q[k];
        }
    }
}

// Anisotropic items' tensor (6) and tensor x position (3), float as stored.
void port_get_aniso_items(void* hp, float* T, float* TX) {
    PortHandle* h = (PortHandle*)hp;
    if (h->metric != 2) return;
    auto* x = static_cast<Engine<AnisoMetric>*>(h->eng);
    for (idt i = 0; i < x->n_items(); i++) {
        for (int k = 0; k < 6; k++) T[6 * i + k] = x->metric.items[i].T[k];
        for (int k = 0; k < 3; k++) TX[3 * i + k] = x->metric.items[i].TX[k];
    }
}

int port_clean(void* hp) { return ((PortHandle*)hp)->eng->clean_clustering(); }
int port_fill_holes(void* hp) { return ((PortHandle*)hp)->eng->fill_holes(); }
int port_connexity_problem(void* hp, long long item, int cluster) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const int save = e->connexity;
    e->connexity = 1;
    const int r = e->connexity_problem(item, cluster);
    e->connexity = save;
    return r;
}

// Topology in the reference's numbering: number of edges; fills edge endpoints
// (2E, may be null) and the CSR of vertex rings (row N+1, col 2E; may be null).
long long port_topology(void* hp, int* edge_v, int* row, int* col) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const Mesh& m = e->mesh;
    if (edge_v)
        for (idt i = 0; i < m.n_edges(); i++) { edge_v[2 * i] = (int)m.ev1[i]; edge_v[2 * i + 1] = (int)m.ev2[i]; }
    if (row && col) {
        idt p = 0;
        for (idt v = 0; v < m.nV; v++) {
            row[v] = (int)p;
            for (idt ed : m.ring[v]) col[p++] = (int)(m.ev1[ed] == v ? m.ev2[ed] : m.ev1[ed]);
        }
        row[m.nV] = (int)p;
    }
    return m.n_edges();
}

// Statistics of the last run: loops, convergences, total moves.
void port_stats(void* hp, int* loops, int* convergences, long long* moves) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    *loops = e->n_loops; *convergences = e->stat_convergences; *moves = e->stat_moves;
}

// BuildDelaunayTriangulation for vertex clustering (vtkDiscreteRemeshing.h:1003-1152
// without display and manifold repair): output vertex k = cluster centroid (empty
// clusters take the first non-empty cluster's), one triangle per input face whose
// three labels are distinct and valid, duplicates (same vertex set) rejected.
// Returns the triangle count; tris (3F) and verts (3K) may be null.
long long port_dual_mesh(void* hp, int* tris, double* verts) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const Mesh& m = e->mesh;
    if (verts) {
        int valid = 0;
        for (int k = 0; k < e->K; k++) if (e->sizes[k] > 0) { valid = k; break; }
        for (int k = 0; k < e->K; k++) {
            double S[3], W, Q[9], c[3];
            e->cluster_accum(e->sizes[k] == 0 ? valid : k, S, &W, Q, c);
            verts[3 * k] = c[0]; verts[3 * k + 1] = c[1]; verts[3 * k + 2] = c[2];
        }
    }
    std::vector<std::vector<std::pair<int, int>>> adj(e->K);  // face lookup by smallest vertex
    long long count = 0;
    for (idt f = 0; f < m.nF; f++) {
        int cl[3]; int n = 0;
        for (int j = 0; j < 3; j++) {
            const int c = e->labels[m.F[3 * f + j]];
            if (c >= e->K) continue;
            bool dup = false;
            for (int t = 0; t < n; t++) if (cl[t] == c) dup = true;
            if (!dup) cl[n++] = c;
        }
        if (n != 3) continue;
        int s[3] = {cl[0], cl[1], cl[2]};
        std::sort(s, s + 3);
        bool exists = false;
        for (auto& pr : adj[s[0]]) if (pr.first == s[1] && pr.second == s[2]) { exists = true; break; }
        if (exists) continue;
        adj[s[0]].push_back({s[1], s[2]});
        if (tris) { tris[3 * count] = cl[0]; tris[3 * count + 1] = cl[1]; tris[3 * count + 2] = cl[2]; }
        count++;
    }
    return count;
}

// The coarse surface of BuildDelaunayTriangulation (vtkDiscreteRemeshing.h:1003-1132)
// for vertex clustering: a face per input face whose clusters are three distinct valid
// ones (GetDualItemNeighbourClusters, :956-984; AddFace skips a face already present,
// :990-999), then, under ForceManifold, an edge (without face) between every pair of
// adjacent clusters not yet joined (:1114-1132).
static void dual_surface(const EngineBase* e, Mesh& d, bool force_manifold) {
    const Mesh& m = e->mesh;
    d.start(e->K);
    for (idt f = 0; f < m.nF; f++) {
        int cl[3];
        int n = 0;
        for (int j = 0; j < 3; j++) {
            const int c = e->labels[m.F[3 * f + j]];
            if (c >= e->K) continue;
            bool dup = false;
            for (int t = 0; t < n; t++) if (cl[t] == c) dup = true;
            if (!dup) cl[n++] = c;
        }
        if (n != 3) continue;
        if (d.is_face(cl[0], cl[1], cl[2]) < 0) d.add_face(cl[0], cl[1], cl[2]);
    }
    if (!force_manifold) return;
    for (idt i = 0; i < m.n_edges(); i++) {
        const int c1 = e->labels[m.ev1[i]], c2 = e->labels[m.ev2[i]];
        if (c1 != c2 && c1 >= 0 && c1 < e->K && c2 >= 0 && c2 < e->K && d.is_edge(c1, c2) < 0) d.add_edge(c1, c2, -1);
    }
}

// vtkIdList::DeleteId: every occurrence removed, the last id taking the freed slot
static void delete_id(std::vector<int>& v, int id) {
    size_t i = 0;
    while (i < v.size()) {
        if (v[i] == id) { v[i] = v.back(); v.pop_back(); }
        else i++;
    }
}

// DetectNonManifoldOutputVertices (vtkDiscreteRemeshing.h:165-383): returns the number
// of topology issues; adds the new clusters and sets IsClusterFreezed.
static int detect_nonmanifold(EngineBase* e) {
    Mesh d;
    dual_surface(e, d, true);
    const int K0 = e->K;
    std::vector<std::vector<int>> items(K0);
    for (int c = 0; c < K0; c++) e->frozen[c] = 1;
    for (idt i = 0; i < e->n_items(); i++) {
        const int c = e->labels[i];
        if (c >= 0 && c < K0) items[c].push_back((int)i);
    }
    int issues = 0;
    std::vector<int> with_issues;
    std::vector<idt> cl;
    for (int c = 0; c < K0; c++) {
        if (d.is_vertex_manifold(c)) continue;
        if (items[c].empty()) continue;
        bool problem = true;
        for (int it : items[c])
            if (!e->mesh.is_vertex_manifold(it)) { problem = false; break; }
        if (!problem) continue;
        issues++;
        with_issues.push_back(c);
        e->frozen[c] = 0;
        d.vertex_neighbours(c, cl);
        for (idt x : cl) e->frozen[x] = 0;
    }
    std::vector<idt> il;
    for (int c : with_issues) {
        e->add_cluster();
        const int nc = e->K - 1;
        items.emplace_back();
        if (items[c].size() > 1) {
            const int it = items[c][0];
            e->labels[it] = nc;
            items[nc].push_back(it);
            delete_id(items[c], it);
            continue;
        }
        const int it = items[c][0];
        e->mesh.vertex_neighbours(it, il);   // GetItemNeighbours (vtkVerticesProcessing.h)
        bool found = false;
        for (idt nb : il) {
            // a cluster added in this pass holds one item; labels >= K0 are unassigned
            // items, which the reference never meets here (MinimizeEnergy fills holes)
            const int ncl = e->labels[nb];
            if (ncl < 0 || ncl >= K0) continue;
            if (items[ncl].size() > 1) {
                e->labels[nb] = nc;
                delete_id(items[ncl], (int)nb);
                items[nc].push_back((int)nb);
                found = true;
                break;
            }
        }
        if (!found) {
            e->remove_last_cluster();
            items.pop_back();
        }
    }
    e->recompute_sizes();
    return issues;
}

// One detection pass on the handle's clustering; *k_out = the new K.
int port_detect_nonmanifold(void* hp, int* k_out) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const int n = detect_nonmanifold(e);
    *k_out = e->K;
    return n;
}

// SetFixedClusters (vtkUniformClustering.h:134): before port_init, so that the
// initial sampling places the fixed items
void port_set_fixed(void* hp, int n, const int* ids) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    e->fixed.assign(ids, ids + n);
}

// GetCluster(c)->AnchorItem = anchors[c] for c < n (QEM only, as ACVDQ.cxx:333-334
// does); -1 for a metric without anchors
int port_set_anchors(void* hp, int n, const int* anchors) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    for (int c = 0; c < n; c++)
        if (!e->set_anchor(c, anchors[c])) return -1;
    return 0;
}

void port_set_frozen(void* hp, const unsigned char* in) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    for (int k = 0; k < e->K; k++) e->frozen[k] = in[k] ? 1 : 0;
}

// MinimizeEnergy again on the current clustering (the ForceManifold re-entry)
void port_minimize(void* hp) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    e->connexity = 0;
    e->minimize_energy();
}

void port_get_frozen(void* hp, unsigned char* out) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    for (int k = 0; k < e->K; k++) out[k] = e->frozen[k];
}

// IsVertexManifold of every vertex of the coarse surface (ForceManifold edges included)
// and of the input mesh.
void port_manifold_flags(void* hp, unsigned char* dual, unsigned char* input) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    Mesh d;
    dual_surface(e, d, true);
    if (dual) for (int c = 0; c < e->K; c++) dual[c] = d.is_vertex_manifold(c) ? 1 : 0;
    if (input) for (idt i = 0; i < e->n_items(); i++) input[i] = e->mesh.is_vertex_manifold(i) ? 1 : 0;
}

// Remesh()'s ForceManifold loop (vtkDiscreteRemeshing.h:937-950) after ProcessClustering:
// detect, then MinimizeEnergy without the connectivity constraint, until no issue is
// left or max_rounds passes ran.  Returns the passes that found issues.
int port_force_manifold(void* hp, int max_rounds) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    int rounds = 0;
    while (rounds < max_rounds && detect_nonmanifold(e)) {
        rounds++;
        e->connexity = 0;
        e->minimize_energy();
    }
    return rounds;
}

int port_get_k(void* hp) { return ((PortHandle*)hp)->eng->K; }

// FixMeshBoundaries (vtkDiscreteRemeshing.h:426-579), pass for pass over the whole edge
// table: the new output vertices (numbered from K, float-rounded as the output's float
// vtkPoints stores them) and the faces it adds.  Returns the face count; *n_pts = the
// vertex count.  pts / faces may be null (counting call).
long long port_fix_mesh_boundaries(void* hp, double* pts, int* faces, long long* n_pts) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const Mesh& m = e->mesh;
    const idt ne = m.n_edges();
    std::vector<idt> np(ne, -2);   // EdgesNewPoint
    std::vector<double> P;
    std::vector<int> F;
    const int K = e->K;
    int nnew = 0;
    auto is_boundary = [&](idt i) { return m.poly2[i] < 0 && m.poly1[i] >= 0; };
    for (idt i = 0; i < ne; i++) {
        if (!is_boundary(i)) continue;
        const idt v1 = m.ev1[i], v2 = m.ev2[i];
        const int c1 = e->labels[v1], c2 = e->labels[v2];
        if (c1 == c2) continue;
        double P1[3], P2[3];
        m.point(v1, P1);
        m.point(v2, P2);
        for (int q = 0; q < 3; q++) P.push_back((double)(float)(0.5 * (P1[q] + P2[q])));
        np[i] = K + nnew++;
        F.insert(F.end(), {(int)np[i], c1, c2});
    }
    std::vector<idt> elist;
    for (idt i = 0; i < ne; i++) {
        if (np[i] >= 0 || !is_boundary(i)) continue;
        const int cluster = e->labels[m.ev1[i]];
        std::queue<idt> q;
        q.push(i);
        elist.clear();
        while (!q.empty()) {
            const idt edge = q.front();
            q.pop();
            if (np[edge] == -2) {
                np[edge] = -1;
                for (idt v : {m.ev1[edge], m.ev2[edge]})
                    for (idt j : m.ring[v])
                        if (m.poly2[j] < 0) q.push(j);
            } else if (np[edge] >= 0) {
                if (std::find(elist.begin(), elist.end(), edge) == elist.end()) elist.push_back(edge);
            }
        }
        if (elist.size() >= 2) F.insert(F.end(), {cluster, (int)np[elist[0]], (int)np[elist[1]]});
    }
    std::vector<idt> nl;
    for (idt v = 0; v < m.nV; v++) {
        // GetNumberOfBoundaries as the reference writes it: Edges[i] for i < valence
        int nb = 0;
        for (idt i = 0; i < (idt)m.ring[v].size(); i++) if (m.poly2[i] < 0) nb++;
        if (nb / 2 <= 0) continue;
        nl.clear();
        for (idt j : m.ring[v])
            if (np[j] >= 0 && std::find(nl.begin(), nl.end(), np[j]) == nl.end()) nl.push_back(np[j]);
        if (nl.size() > 1) F.insert(F.end(), {e->labels[v], (int)nl[0], (int)nl[1]});
    }
    if (pts) std::memcpy(pts, P.data(), P.size() * sizeof(double));
    if (faces) std::memcpy(faces, F.data(), F.size() * sizeof(int));
    *n_pts = nnew;
    return (long long)F.size() / 3;
}

// Curvature of vertex clustering (vtkDiscreteRemeshing::SamplingPreProcessing,
// DiscreteRemeshing/vtkDiscreteRemeshing.h:630-637 -> Common/vtkCurvatureMeasure.cxx,
// polynomial fitting, vertices, 3-ring).
//
// Faces of the 3-ring of vertex v (vtkNeighbourhoodComputation::ComputeNRingCells,
// Common/vtkNeighbourhoodComputation.cxx:38-100): v's own faces first, then ring by
// ring the faces of the edges of every not yet visited vertex, in ring order.
static void nring_faces(const Mesh& m, idt v, int rings, std::vector<idt>& faces, std::vector<char>& ftag,
                        std::vector<char>& vtag, std::vector<idt>& touched_f, std::vector<idt>& touched_v) {
    m.vertex_faces(v, faces);
    for (idt f : faces) { ftag[f] = 1; touched_f.push_back(f); }
    std::vector<idt> cur{v}, next;
    for (int r = 0; r < rings; r++) {
        next.clear();
        for (idt u : cur) {
            if (vtag[u]) continue;
            vtag[u] = 1;
            touched_v.push_back(u);
            for (idt e : m.ring[u]) {
                next.push_back(m.ev1[e] == u ? m.ev2[e] : m.ev1[e]);
                const idt f1 = m.poly1[e], f2 = m.poly2[e];
                if (f1 >= 0) {
                    if (!ftag[f1]) { faces.push_back(f1); ftag[f1] = 1; touched_f.push_back(f1); }
                    if (f2 >= 0 && !ftag[f2]) { faces.push_back(f2); ftag[f2] = 1; touched_f.push_back(f2); }
                }
            }
        }
        std::swap(cur, next);
    }
}

// vtkSurface::GetCellMassProperties for a triangle (Common/vtkSurface.cxx:1380-1419)
static void face_mass(const Mesh& m, idt f, double& area, double* bary) {
    double p1[3], p2[3], p3[3];
    m.point(m.F[3 * f], p1); m.point(m.F[3 * f + 1], p2); m.point(m.F[3 * f + 2], p3);
    area = 0;
    bary[0] = bary[1] = bary[2] = 0;
    const double a2 = rmath::tri_area(p1, p2, p3);
    for (int i = 0; i < 3; i++) bary[i] += a2 * (p1[i] + p2[i] + p3[i]) / 3.0;
    area += a2;
    if (area > 0)
        for (int i = 0; i < 3; i++) bary[i] /= area;
}

// vtkSinglePolynomialMeasure::ComputeFitting (Common/vtkCurvatureMeasure.cxx:188-505):
// local frame from the area-weighted mean normal, least-squares quadratic height
// field z = q0 + q1 x + q2 y + q3 x^2 + q4 xy + q5 y^2 through the face barycentres,
// shape operator from the fundamental forms, its eigen-decomposition; returns
// sqrt(k1^2 + k2^2) and writes the two principal directions scaled by sqrt|k|,
// the larger |k| first.
static double fit_curvature(const Mesh& m, const std::vector<idt>& fl, double info[6]) {
    double sarea = 0, origin[3] = {0, 0, 0}, frame[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (idt f : fl) {
        double p1[3], p2[3], p3[3], nrm[3], area, bary[3];
        m.point(m.F[3 * f], p1); m.point(m.F[3 * f + 1], p2); m.point(m.F[3 * f + 2], p3);
        rmath::tri_normal(p1, p2, p3, nrm);
        face_mass(m, f, area, bary);
        for (int k = 0; k < 3; k++) {
            origin[k] += area * bary[k];
            frame[0][k] += area * nrm[k];
        }
        sarea += area;
    }
    for (int j = 0; j < 3; j++) origin[j] = origin[j] / sarea;
    auto normalize = [](double* a) {
        const double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (n != 0.0) { a[0] /= n; a[1] /= n; a[2] /= n; }
    };
    auto cross = [](const double* a, const double* b, double* c) {
        const double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
        c[0] = x; c[1] = y; c[2] = z;
    };
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    normalize(frame[0]);
    for (int k = 0; k < 3; k++) frame[2][k] = frame[0][k];
    frame[1][1] = frame[2][0]; frame[1][2] = frame[2][1]; frame[1][0] = frame[2][2];
    cross(frame[1], frame[2], frame[0]);
    normalize(frame[0]);
    cross(frame[2], frame[0], frame[1]);
    for (int i = 0; i < 6; i++) info[i] = 0;
    const int nf = (int)fl.size();
    if (nf <= 6) return 0;
    std::vector<double> V((size_t)nf * 6), Z(nf);
    double h = 0;
    for (int j = 0; j < nf; j++) {
        double area, bary[3];
        face_mass(m, fl[j], area, bary);
        for (int k = 0; k < 3; k++) bary[k] -= origin[k];
        const double x = dot(bary, frame[0]), y = dot(bary, frame[1]), z = dot(bary, frame[2]);
        double* r = &V[(size_t)j * 6];
        r[0] = 1.0; r[1] = x; r[2] = y; r[3] = x * x; r[4] = x * y; r[5] = y * y;
        Z[j] = z;
        h += std::sqrt(x * x + y * y);
    }
    h = h / ((double)nf);
    for (int j = 0; j < nf; j++) {
        double* r = &V[(size_t)j * 6];
        r[1] /= h; r[2] /= h; r[3] /= h * h; r[4] /= h * h; r[5] /= h * h;
    }
    // normal equations (upper half, then mirrored), the reference's SolveLeastSquares (:508-616)
    double xxt[6][6] = {}, xxti[6][6] = {}, xyt[6] = {}, q[6];
    for (int k = 0; k < nf; k++) {
        const double* r = &V[(size_t)k * 6];
        for (int i = 0; i < 6; i++) {
            for (int j = i; j < 6; j++) xxt[i][j] += r[i] * r[j];
            xyt[i] += r[i] * Z[k];
        }
    }
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < i; j++) xxt[i][j] = xxt[j][i];
    double* xr[6]; double* xir[6];
    for (int i = 0; i < 6; i++) { xr[i] = xxt[i]; xir[i] = xxti[i]; }
    if (!rmath::lu_invert(xr, xir, 6)) return 0;
    for (int i = 0; i < 6; i++) {
        q[i] = 0.0;
        for (int k = 0; k < 6; k++) q[i] += xxti[i][k] * xyt[k];
    }
    q[1] /= h; q[2] /= h; q[3] /= h * h; q[4] /= h * h; q[5] /= h * h;
    const double E = 1.0 + q[1] * q[1], F = q[1] * q[2], G = 1.0 + q[2] * q[2];
    const double e = 2.0 * q[3] / std::sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    const double ff = 2.0 * q[4] / std::sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    const double g = 2.0 * q[5] / std::sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    double A[2][2] = {{E, F}, {F, G}}, B[2][2];
    double* ar[2] = {A[0], A[1]}; double* br[2] = {B[0], B[1]};
    if (!rmath::lu_invert(ar, br, 2)) return 0;
    A[0][0] = -(e * B[0][0] + ff * B[1][0]);
    A[1][0] = -(e * B[0][1] + ff * B[1][1]);
    A[0][1] = -(ff * B[0][0] + g * B[1][0]);
    A[1][1] = -(ff * B[0][1] + g * B[1][1]);
    double ev[2], evec[2][2];
    double* vr[2] = {evec[0], evec[1]};
    if (!rmath::jacobi_upper(ar, 2, ev, vr)) return 0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 3; k++) info[k + 3 * j] += std::sqrt(std::fabs(ev[j])) * evec[i][j] * frame[i][k];
    if (std::fabs(ev[0]) < std::fabs(ev[1]))
        for (int i = 0; i < 3; i++) std::swap(info[i], info[i + 3]);
    return std::sqrt(ev[0] * ev[0] + ev[1] * ev[1]);
}

// Per-vertex curvature indicator and principal directions (6 per vertex, float as
// the reference stores them) of the vertices [v0, v1); outputs indexed by vertex.
// The reference's vtkCurvatureMeasure deals the vertices to its threads the same way
// (each vertex is independent, Common/vtkCurvatureMeasure.cxx:625-718).
void port_curvature_range(void* hp, long long v0, long long v1, double* indicator, float* principal_dirs) {
    const Mesh& m = ((PortHandle*)hp)->eng->mesh;
    std::vector<char> ftag(m.nF, 0), vtag(m.nV, 0);
    std::vector<idt> faces, tf, tv;
    for (idt v = v0; v < v1; v++) {
        faces.clear(); tf.clear(); tv.clear();
        nring_faces(m, v, 3, faces, ftag, vtag, tf, tv);
        double info[6];
        indicator[v] = fit_curvature(m, faces, info);
        for (int i = 0; i < 6; i++) principal_dirs[6 * v + i] = (float)info[i];
        for (idt f : tf) ftag[f] = 0;
        for (idt u : tv) vtag[u] = 0;
    }
}

// vtkSurface::Subdivide (Common/vtkSurface.cxx:605-677): the old points, then one
// midpoint per active edge in edge order (stored in a float vtkPoints, hence the
// rounding), then four faces per active face; VerticesParent1/2 of the new vertex
// nV + e are the edge's endpoints.  With an indicator, the parent interpolation of
// vtkDiscreteRemeshing::SamplingPreProcessing (vtkDiscreteRemeshing.h:731-745):
// old values copied, new (ind[p1] + ind[p2]) * 0.5.  Returns the number of output
// faces; out_pts: 3 (nV + nE), out_tri: 12 nF, p1/p2: nE, ind_out: nV + nE.
long long port_subdivide(long long nv, const double* pts, long long nf, const int* tri, double* out_pts,
                         int* out_tri, int* p1, int* p2, const double* ind, double* ind_out, double* seconds) {
    Mesh m;
    m.build(nv, pts, nf, tri);
    // the reference subdivides a vtkSurface whose edge table exists: time from here
    const auto t0 = std::chrono::steady_clock::now();
    const idt ne = m.n_edges();
    std::vector<idt> child(ne, -1);
    idt nout = 0;
    auto add_vertex = [&](const double* P) {
        for (int c = 0; c < 3; c++) out_pts[3 * nout + c] = (double)(float)P[c];
        return nout++;
    };
    for (idt i = 0; i < nv; i++) {
        double P[3];
        m.point(i, P);
        add_vertex(P);
        if (ind) ind_out[i] = ind[i];
    }
    for (idt e = 0; e < ne; e++) {
        const idt v1 = m.ev1[e], v2 = m.ev2[e];
        double P1[3], P2[3], P[3];
        m.point(v1, P1);
        m.point(v2, P2);
        P[0] = 0.5 * (P1[0] + P2[0]);
        P[1] = 0.5 * (P1[1] + P2[1]);
        P[2] = 0.5 * (P1[2] + P2[2]);
        const idt v3 = add_vertex(P);
        child[e] = v3;
        p1[e] = (int)v1;
        p2[e] = (int)v2;
    }
    // the reference interpolates in increasing vertex id; a new vertex's parents are
    // old vertices of this level
    if (ind)
        for (idt i = nv; i < nv + ne; i++)
            ind_out[i] = (ind_out[p1[i - nv]] + ind_out[p2[i - nv]]) * 0.5;
    long long of = 0;
    for (idt f = 0; f < nf; f++) {
        const idt V1 = m.F[3 * f], V2 = m.F[3 * f + 1], V3 = m.F[3 * f + 2];
        if (V1 == V2) continue;  // inactive face
        const int V4 = (int)child[m.is_edge(V1, V2)];
        const int V5 = (int)child[m.is_edge(V2, V3)];
        const int V6 = (int)child[m.is_edge(V3, V1)];
        const int t[12] = {(int)V1, V4, V6, V4, (int)V2, V5, V5, (int)V3, V6, V4, V5, V6};
        for (int j = 0; j < 12; j++) out_tri[12 * of + j] = t[j];
        of++;
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 4 * of;
}

void port_curvature(void* hp, double* indicator, float* principal_dirs) {
    port_curvature_range(hp, 0, ((PortHandle*)hp)->eng->mesh.nV, indicator, principal_dirs);
}

// ACVD's quadric post-placement (DiscreteRemeshing/Examples/ACVD.cxx:217-291): per
// cluster, the unweighted plane quadrics (FullQuadric = false) of all faces adjacent to
// each of its items (a face once per item, items in increasing id, faces in the
// vertex's ring order); the output vertex -- the cluster centroid, or the first
// non-empty cluster's for an empty one (BuildDelaunayTriangulation,
// vtkDiscreteRemeshing.h:1024-1033) -- moved by ComputeRepresentativePoint with
// `level` singular values.  verts: 3K.
void port_post_placement(void* hp, int level, double* verts) {
    EngineBase* e = ((PortHandle*)hp)->eng;
    const Mesh& m = e->mesh;
    std::vector<double> Q(9 * (size_t)e->K, 0.0);
    std::vector<idt> fl;
    for (idt i = 0; i < m.nV; i++) {
        const int c = e->labels[i];
        if (c < 0 || c >= e->K) continue;
        m.vertex_faces(i, fl);
        for (idt f : fl) m.add_triangle_quadric(&Q[9 * (size_t)c], f);
    }
    int valid = 0;
    for (int k = 0; k < e->K; k++) if (e->sizes[k] > 0) { valid = k; break; }
    for (int k = 0; k < e->K; k++) {
        double S[3], W, Qc[9], c[3];
        e->cluster_accum(e->sizes[k] == 0 ? valid : k, S, &W, Qc, c);
        representative_point(&Q[9 * (size_t)k], c, level);
        verts[3 * k] = c[0]; verts[3 * k + 1] = c[1]; verts[3 * k + 2] = c[2];
    }
}

}  // extern "C"

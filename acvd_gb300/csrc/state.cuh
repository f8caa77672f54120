// Device-side data layout of one clustering context and the launchers of the
// kernels that operate on it.  All arrays live in HBM; kernels get raw pointers.
//
// Items (one per mesh vertex), float32:
//   xw[i] = (x, y, z, w)                      all metrics
//   qa[i] = (A00, A01, A02, A11), qb[i] = (A12, A22)
//                                             quadric metrics: A = sum over the
//                                             adjacent faces of n n^T (unit normals);
//                                             the linear part of the reference's
//                                             quadric is b_i = A_i x_i exactly, since
//                                             x_i lies on every adjacent face plane
//   ta[i] = (T00, T01, T02, T11), tb[i] = (T12, T22)   anisotropic tensor
//
// Clusters: compensated (double-float) accumulators, acc[k * acc_stride + j]:
//   j = 0..2 S = sum w x, 3 W = sum w, 4..9 A, 10..12 b = sum A_i x_i,
//   13..18 T = sum T_i, 19..21 u = sum T_i x_i
// and a float32 evaluation record derived from them in FP64 (update_cluster),
// ev[k * ev_stride + j] (float4):
//   0 (m, W)  m = S / W          1 (delta, P)  placed vertex c = m + delta, P = W |delta|^2
//   2 (r, 0)  r = b - A m        3 (A00 A01 A02 A11)   4 (A12 A22 0 0)
//   5 (T00 T01 T02 T11)          6 (T12 T22 g0 g1)     7 (g2 0 0 0)   g = u - T c
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace acvd {

enum Metric { kIso = 0, kQEM = 1, kAniso = 2 };

// Matching rounds per colour step (claim epochs: colour * kRounds + round, at
// most 64 colours, so epochs fit the claim word's 8-bit field).
constexpr int kRounds = 4;

// A cluster taken by a commit keeps this value for the rest of the colour step: it
// is below every claim of the step's rounds (same or older epoch; a real claim's
// priority is never 0) and above every claim of the following steps, so claims need
// resetting once per sweep only.
ACVD_HD unsigned long long claim_taken(int color) {
    return make_claim((unsigned)(color * kRounds + kRounds - 1), 0u, 0u);
}

template <int M> struct Layout;
template <> struct Layout<kIso> { static constexpr int acc = 4, ev = 1; };
template <> struct Layout<kQEM> { static constexpr int acc = 13, ev = 5; };
template <> struct Layout<kAniso> { static constexpr int acc = 22, ev = 8; };

inline int acc_stride(int m) { return m == kIso ? 4 : (m == kQEM ? 13 : 22); }
inline int ev_stride(int m) { return m == kIso ? 1 : (m == kQEM ? 5 : 8); }

// Mutable run flags read by the kernels from device memory, so that one captured
// sweep graph serves every phase of the minimisation.
struct RunFlags {
    int constrained;   // quadric placement active (QEM after the unconstrained phase; always for aniso)
    int connexity;     // local connectivity constraint active
    int level;         // number of eigenvalues the placement may invert (0..3)
    float thr;         // relative eigenvalue threshold (1e-3)
};

// Counters written by the kernels.
enum Counter {
    kCntMoves = 0,       // accepted moves in the current sweep
    kCntCand = 1,        // candidate moves proposed
    kCntBoundary = 2,    // boundary items evaluated
    kCntTargets = 3,     // (item, destination cluster) energy evaluations
    kCntVisited = 4,     // items visited by the evaluation kernels
    kCntSlots = 5,       // ring slots read by the evaluation kernels
    kCntChanged = 6,     // generic "something changed" flag / count
    kCntError = 7,       // device-side check failures
    kCntDisconnected = 8,
    kCntAssigned = 9,
    kCntReverted = 10,   // commits undone because the pair's energy did not decrease
    kCntScreened = 11,   // visited items whose boundary flag sent them to the ring screen
    kCntCached = 12,     // ring screens answered from the item's screen cache
    kNumCounters = 16
};

// The counters are striped over kStripes 128-byte lines: a block adds into the
// stripe of its index, so tens of thousands of warps do not serialise on one
// address; the host sums the stripes.
constexpr int kStripes = 32;
constexpr int kCounterWords = kStripes * kNumCounters;
__device__ __forceinline__ unsigned long long* ctr(unsigned long long* counters, int which) {
    return counters + (blockIdx.x & (kStripes - 1)) * kNumCounters + which;
}

// Bounds checks of device-side indices, compiled in with -DACVD_DEVICE_CHECKS (the
// build that stands in for a sanitizer): a failed check counts in kCntError, the access
// is skipped and the host fails the call with ACVD_ERR_DEVICE_CHECK.  Without the flag
// the checks compile away.
#ifdef ACVD_DEVICE_CHECKS
#define ACVD_VALID(st, cond) ((cond) || (atomicAdd(ctr((st).counters, kCntError), 1ull), false))
#else
#define ACVD_VALID(st, cond) true
#endif

// Packed cached screen (16 bytes).  Cluster ids below 2^24 (kCacheClusters; a
// clustering with more clusters never caches), e = evaluation sweep + 1 below 2^28
// (0 for "never evaluated without a proposal"):
//   x = L  | meta << 24 | (e >> 24) << 28      meta = count | 4 if the connectivity
//   y = t0 | (e & 0xff) << 24                        test is known | 8 if it passed
//   z = t1 | ((e >> 8) & 0xff) << 24
//   w = t2 | ((e >> 16) & 0xff) << 24
// Unused targets are 0.  The evaluation sweep is kept here as well as in evald, and
// every write of evald for an item whose screen is cached writes both.
constexpr int kCacheClusters = 1 << 24;
constexpr int kCacheSweeps = (1 << 28) - 2;   // evaluation sweeps a record can hold
struct Screen {
    int L, t[3], n, ev;
    bool conn_known, conn_ok;
};
__host__ __device__ inline int4 pack_screen(int L, int t0, int t1, int t2, int meta, int ev) {
    const unsigned e = (unsigned)(ev + 1);
    return make_int4((int)((unsigned)L | ((unsigned)meta << 24) | ((e >> 24) << 28)),
                     (int)((unsigned)t0 | ((e & 0xffu) << 24)), (int)((unsigned)t1 | (((e >> 8) & 0xffu) << 24)),
                     (int)((unsigned)t2 | (((e >> 16) & 0xffu) << 24)));
}
__host__ __device__ inline Screen unpack_screen(int4 c) {
    const unsigned m = (1u << 24) - 1u;
    const unsigned x = (unsigned)c.x, y = (unsigned)c.y, z = (unsigned)c.z, w = (unsigned)c.w;
    Screen r;
    r.L = (int)(x & m);
    r.t[0] = (int)(y & m);
    r.t[1] = (int)(z & m);
    r.t[2] = (int)(w & m);
    const unsigned meta = (x >> 24) & 15u;
    r.n = (int)(meta & 3u);
    r.conn_known = (meta & 4u) != 0;
    r.conn_ok = (meta & 8u) != 0;
    const unsigned e = (y >> 24) | ((z >> 24) << 8) | ((w >> 24) << 16) | ((x >> 28) << 24);
    r.ev = (int)e - 1;
    return r;
}
// the record with its evaluation sweep replaced
__host__ __device__ inline int4 screen_with_ev(int4 c, int ev) {
    const unsigned m = (1u << 24) - 1u;
    const unsigned e = (unsigned)(ev + 1);
    return make_int4((int)(((unsigned)c.x & ((1u << 28) - 1u)) | ((e >> 24) << 28)),
                     (int)(((unsigned)c.y & m) | ((e & 0xffu) << 24)),
                     (int)(((unsigned)c.z & m) | (((e >> 8) & 0xffu) << 24)),
                     (int)(((unsigned)c.w & m) | (((e >> 16) & 0xffu) << 24)));
}

// Sweep bookkeeping on the device (one captured graph serves every sweep):
// `sweep` counts sweeps, `floor` is the sweep after which every cluster counts as
// modified (the reference's SetAllClustersToModified, vtkUniformClustering.h:717-722).
struct SweepState {
    int sweep;
    int floor;
};

// Work list of the split evaluation (screen_kernel -> eval_list_kernel): stripes
// and the items one screen block covers; stripe s of a class of `count` items holds
// its entries at [s * work_cap(count), (s + 1) * work_cap(count)).
constexpr int kWorkStripes = 16;
constexpr int kScreenTile = 4096;
__host__ __device__ inline int64_t work_cap(int64_t count) {
    const int64_t nb = (count + kScreenTile - 1) / kScreenTile;
    return ((nb + kWorkStripes - 1) / kWorkStripes) * kScreenTile;
}

struct DevState {
    int64_t n;        // items
    int k;            // clusters; label k = null (unassigned)
    const int* row;   // CSR of vertex rings (reference ring order)
    const int* col;
    const unsigned* adj;        // per CSR slot: which ring slots are adjacent to this neighbour
    const float4* xw;
    const float4* qa;
    const float2* qb;
    const float4* ta;
    const float2* tb;
    int* label;
    int* size;
    unsigned long long* claim;
    df* acc;
    float4* ev;
    double* energy;
    unsigned long long* counters;
    const RunFlags* flags;
    SweepState* sweep;     // sweep counter / invalidation floor
    int* stamp;            // per cluster: sweep of its last modification
    int* evald;            // per item: sweep of its last evaluation without a proposal (-1: none)
    int* cand_list;        // compact list of proposals (colour-list positions) of the current step
    unsigned* cand_count;  // per colour: number of proposals
    // relaxed steps: per cluster, exact fixed-point sums of the committed moves'
    // contributions (order-independent, hence deterministic with atomics)
    long long* fx_delta;   // K x acc stride
    const float4* fx_pow;  // per accumulator component: fixed-point scale 2^e as two float factors
                           // (x, y) and their inverses (z, w)
    int* out_cnt;          // proposals leaving the cluster in this step
    int* in_done;          // committed moves into the cluster
    int* out_done;         // committed moves out of the cluster
    // per item: 0 = certainly interior (every ring label equals its own), 1 = maybe
    // on a cluster boundary, 2 = on a boundary with its screen in tcache.  A commit
    // sets 1 on the moved item and its ring; the ring screen sets 0 when it finds the
    // item interior, 2 when it caches the screen.  The reference keeps only boundary
    // edges in its queue and re-queues a moved item's ring
    // (vtkUniformClustering.h:858-872, 971, 985).
    unsigned char* bflag;
    // per item with bflag 2: its packed cached screen (pack_screen: its cluster, its
    // distinct neighbour clusters in ring order, the connectivity bits and a copy of
    // its evaluation sweep), 16 bytes so that a cached screen reads one record.
    // Valid while no label in the ring changes.
    int4* tcache;
    // per item, the first 8 ring neighbours (two int4, ring order, -1 padded; slot
    // 7 = -2 when the ring is longer than 8, which then is read from row / col)
    const int4* ring8;
    // internal item order (colour classes contiguous): original vertex id of
    // each item, and the item of each original vertex id
    const int* orig;
    const int* inv;
    // per cluster: 1 = frozen (IsClusterFreezed, vtkUniformClustering.h:912-915): no
    // item leaves it and none joins it, except unassigned items; null: none frozen
    const unsigned char* frozen;
    // per cluster, QEM metric: the item of its anchor vertex (Cluster::AnchorItem,
    // vtkQEMetricForClustering.h:127-128; -1 = none) and that vertex's coordinates;
    // null: no anchored cluster
    const int* anchor;
    const double* anchor_xyz;
    // fixed items (FixedClusters, vtkUniformClustering.h:134): cluster c < nfixed
    // holds item fixed[c]; cleaning keeps the component that contains it
    const int* fixed;
    int nfixed;
    // split evaluation of large colour classes: the work list (kWorkStripes stripes
    // of work_cap(class size) entries) and its per-(class, stripe) counts; null when
    // no class is split
    int* work = nullptr;
    unsigned* work_count = nullptr;
};

// Persistent sweep kernel: the loop that runs colour sweeps back to back on the
// device between two convergence events.  Host-written fields are marked "in";
// the kernel updates the others (block 0 decides after each sweep, every block
// reads the decision after a grid barrier).
struct LoopState {
    long long early;          // in: items of non-frozen clusters (base of the early-convergence test)
    long long moves;          // out: moves committed by this launch's sweeps
    long long last_moves;     // out: moves of the last sweep
    double e_prev;            // in/out: energy after the previous relaxed sweep
    unsigned long long eval_ns;  // out: device time spent in the evaluation phases
    int sweeps;               // in/out: sweeps of this minimisation so far
    int max_loops;            // in: sweep cap
    int convergences;         // in: convergence events so far
    int relaxed_ok;           // in/out: relaxed sweeps allowed
    int have_prev;            // in/out: e_prev is valid
    int relaxed_run;          // out: relaxed sweeps run by this launch
    int run;                  // out: sweeps run by this launch
    int status;               // out: 0 running, 1 convergence test met, 2 grid barrier gave up
};

// Grid-wide barrier of the persistent kernel (all blocks co-resident: cooperative launch).
struct GridBar {
    unsigned count;           // blocks arrived in the current generation
    unsigned gen;             // generation, bumped by the last block to arrive
    int err;                  // set when a wait gave up
    int pad;
};

// One record per sweep (trace output).
struct SweepLog {
    long long moves;
    double energy;            // relaxed sweeps: the energy after the sweep
    int relaxed;
    int pad;
};

// Arguments of the persistent sweep kernel.
struct SweepRun {
    DevState st;
    const long long* off;     // class offsets (nclasses + 1)
    int nclasses;
    int match_rounds;
    int* cand_dest;
    unsigned* cand_prio;
    LoopState* ls;
    GridBar* bar;
    double* esum;             // energy-sum partials: ceil(K/2048) + ceil(K/2048^2) + 2 doubles
    SweepLog* log;
    int log_cap;
};

// ---- items / topology (topology.cu) ----
cudaError_t launch_ring_adjacency(const int* row, const int* col, int64_t n, unsigned* adj, int* max_deg,
                                  cudaStream_t s);
cudaError_t launch_color_round(const int* row, const int* col, int64_t n, int* color,
                               unsigned long long* remaining, int* max_color, cudaStream_t s);
cudaError_t launch_face_geometry(const double* xyz, const int* tri, int64_t nf, double* farea, double* fnorm,
                                 cudaStream_t s);
cudaError_t launch_vertex_keys(const int* tri, int64_t nf, uint32_t* keys, uint32_t* vals, cudaStream_t s);
cudaError_t launch_segment_offsets(const uint32_t* sorted_keys, int64_t n, uint32_t nkeys, uint32_t* off,
                                   cudaStream_t s);
cudaError_t launch_vertex_items(int metric, int64_t nv, const double* xyz, const uint32_t* vf_row,
                                const uint32_t* vf_face, const double* farea, const double* fnorm,
                                const double* indicator, double gradation, double* wd, double* varea,
                                float4* qa, float2* qb, cudaStream_t s);
cudaError_t launch_mesh_sums(const double* wd, const int64_t* v_off, int nmesh, double* out, cudaStream_t s);
cudaError_t launch_finish_items(int metric, int64_t nv, const double* xyz, const double* wd, const double* vrea,
                                const double* wsum, const int64_t* v_off, int nmesh, double ratio, const float* pdirs,
                                float4* xw, float4* ta, float2* tb, cudaStream_t s);

// ---- internal item order (topology.cu) ----
cudaError_t launch_scatter_inv(const int* perm, int64_t n, int* inv, cudaStream_t s);
cudaError_t launch_perm_degree(const int* row, const int* perm, int64_t n, uint32_t* deg, cudaStream_t s);
cudaError_t launch_perm_ring(const int* row, const int* col, const int* perm, const int* inv, const uint32_t* row_new,
                             int64_t n, int* col_new, cudaStream_t s);
cudaError_t launch_map_ids(const int* in, int64_t m, const int* inv, int* out, cudaStream_t s);
// the uploaded mesh arrays' ids and ring offsets checked on the device (*bad: violations)
cudaError_t launch_validate_mesh(const int* row, const int* col, int64_t n, int64_t ncol, const int* tri,
                                 int64_t ntri, const int* ev, int64_t nev, unsigned* bad, cudaStream_t s);
// gather of labels that also counts those outside [0, k] in *bad
// per cluster c < n: the item of vertex ids[c] (-1 stays -1) and, when xyz_out
// is given, the vertex's coordinates (0 for -1)
cudaError_t launch_anchor_setup(const int* ids, int n, const int* inv, const double* xyz, int* item_out,
                                double* xyz_out, cudaStream_t s);
cudaError_t launch_gather_labels(const int* src, const int* idx, int64_t n, int k, int* dst, unsigned* bad,
                                 cudaStream_t s);
cudaError_t launch_gather_i32(const int* src, const int* idx, int64_t n, int* dst, cudaStream_t s);
cudaError_t launch_gather_f4(const float4* src, const int* idx, int64_t n, float4* dst, cudaStream_t s);
cudaError_t launch_gather_f2(const float2* src, const int* idx, int64_t n, float2* dst, cudaStream_t s);
cudaError_t launch_iota(int64_t n, int* out, cudaStream_t s);
cudaError_t launch_ring8(const int* row, const int* col, int64_t n, int* ring8, cudaStream_t s);

// ---- clustering (cluster.cu) ----
// The sweep kernels take a colour class as the contiguous item range
// [item0, item0 + count) of the internal order.
cudaError_t launch_begin_sweep(const DevState& st, int ncolors, bool reset_claims, cudaStream_t s);
// the grid barrier with one block that never arrives (its wait limit's self-check)
cudaError_t launch_barrier_wait_limit(GridBar* bar, long long max_spins, cudaStream_t s);
// device-side sweep loop (graph WHILE node): set the loop and mode conditions at the
// start, and after each sweep (relaxed: e_now holds the energy after the sweep)
cudaError_t launch_loop_start(const LoopState* ls, const RunFlags* flags, cudaGraphConditionalHandle h_loop,
                              cudaGraphConditionalHandle h_mode, cudaStream_t s);
cudaError_t launch_loop_decide(LoopState* ls, const unsigned long long* counters, const double* e_now,
                               const RunFlags* flags, bool relaxed, cudaGraphConditionalHandle h_loop,
                               cudaGraphConditionalHandle h_mode, cudaStream_t s);
cudaError_t launch_relaxed_step(int metric, const DevState& st, int item0, int64_t count, int color,
                                const int* cand_dest, cudaStream_t s);
cudaError_t launch_fx_scale(int metric, const DevState& st, unsigned* maxbits, cudaStream_t s);
// blocks: 256-thread blocks per SM (3..5, else the defaults); threads: 128 for
// 128-thread blocks at the threads per SM of four 256-thread blocks (else 256)
cudaError_t launch_eval(int metric, const DevState& st, int item0, int64_t count, int color,
                        int* cand_dest, unsigned* cand_prio, bool claims, bool split, int blocks, int threads,
                        cudaStream_t s);
cudaError_t launch_apply(int metric, const DevState& st, int item0, int64_t count, int color, int round,
                         int* cand_dest, const unsigned* cand_prio, cudaStream_t s);
cudaError_t launch_reclaim(const DevState& st, int item0, int64_t count, int color, int round,
                           int* cand_dest, const unsigned* cand_prio, cudaStream_t s);
// Persistent sweep kernel (cooperative launch).  blocks_per_sm: co-resident
// blocks per SM for this metric (0 when the kernel cannot be co-resident).
int sweep_run_blocks_per_sm(int metric);
cudaError_t launch_sweep_run(int metric, const SweepRun& a, int grid, cudaStream_t s);
cudaError_t launch_update_all(int metric, const DevState& st, cudaStream_t s);
cudaError_t launch_cluster_keys(const DevState& st, uint32_t* keys, uint32_t* vals, uint32_t* counts,
                                cudaStream_t s);
cudaError_t launch_reduce_clusters(int metric, const DevState& st, const uint32_t* sorted_items,
                                   const uint32_t* seg_off, const uint32_t* seg_cnt, cudaStream_t s);
cudaError_t launch_comp_init(const DevState& st, int* comp, cudaStream_t s);
cudaError_t launch_comp_step(const DevState& st, int* comp, cudaStream_t s);
// the components in one union-find pass, at most `tries` attempts per link; kCntChanged
// counts links it gave up on (then the propagation above runs instead)
cudaError_t launch_comp_union(const DevState& st, int* comp, int* parent, int tries, cudaStream_t s);
cudaError_t launch_comp_finish(const DevState& st, const int* comp, int* csize, unsigned long long* best,
                               int* multi, cudaStream_t s);
// hole filling over lists of the unassigned items: collect them per colour class
// (class c's list at list[off[c] ...], cnt[c] entries; off: ncolors + 1 class offsets
// on the device), then one round of class c over its list (cap: the class size)
cudaError_t launch_fill_collect(const DevState& st, const int64_t* off, int ncolors, int* list, unsigned* cnt,
                                cudaStream_t s);
cudaError_t launch_fill_list(const DevState& st, const int* list, const unsigned* cnt, int64_t cap, cudaStream_t s);
// every round over the class lists in one block when they hold at most max_items
// items; *err = 1 if the round bound ran out, 2 if the lists were longer (nothing done)
cudaError_t launch_fill_block(const DevState& st, const int* list, const int64_t* off, int ncolors,
                              const unsigned* cnt, unsigned* err, unsigned max_items, cudaStream_t s);
cudaError_t launch_boundary_edges(const int* edge_v, int64_t ne, const int* label, uint32_t* flags,
                                  cudaStream_t s);
cudaError_t launch_compact(const uint32_t* flags, const uint32_t* pos, int64_t n, int* out, cudaStream_t s);
cudaError_t launch_dual_faces(const int* tri, int64_t nf, const int* label, int k, uint32_t* flags,
                              cudaStream_t s);
cudaError_t launch_dual_keys(const int* tri, const int* faces, int64_t m, const int* label, uint32_t* klo,
                             uint32_t* khi, uint32_t* order, cudaStream_t s);
cudaError_t launch_gather_u32(const uint32_t* src, const uint32_t* idx, int64_t m, uint32_t* dst, cudaStream_t s);
cudaError_t launch_dual_unique(const uint32_t* klo, const uint32_t* khi, const uint32_t* order, int64_t m,
                               uint32_t* keep, cudaStream_t s);
cudaError_t launch_dual_write(const int* tri, const int* faces, const int* sel, int64_t t, const int* label,
                              int* out, cudaStream_t s);
cudaError_t launch_centroids(int metric, const DevState& st, double* out, cudaStream_t s);
cudaError_t launch_vertex_quadrics(const double* xyz, const int* tri, const uint32_t* vf_row, const uint32_t* vf_face,
                                   int64_t nv, double* qv, cudaStream_t s);
cudaError_t launch_post_place(const double* qv, const uint32_t* sorted, const uint32_t* seg_off,
                              const uint32_t* seg_cnt, const int* size, int* first, const double* start, int k,
                              int level, double* out, cudaStream_t s);

// ---- curvature (curvature.cu) ----
size_t curvature_face_bytes(int64_t nf);
cudaError_t launch_curvature(const double* xyz, const int* tri, int64_t nv, int64_t nf, int64_t ne,
                             const int* edge_v, const int* edge_int, const uint32_t* vf_row, const uint32_t* vf_face,
                             const int* row, const int* col, const int* perm, const int* inv, int2* poly,
                             int* slot_edge, void* face_work, double* indicator, float* dirs,
                             unsigned long long* overflow, cudaStream_t s);

// ---- midpoint subdivision (subdivide.cu) ----
// One level of vtkSurface::Subdivide over a mesh in the reference's numbering
// (ring CSR and edge list of acvd_build_topology); ind / out_ind may be null.
cudaError_t launch_subdivide(const double* xyz, int64_t nv, const int* tri, int64_t nf, const int* row,
                             const int* col, const int* edge_v, int64_t ne, const double* ind, int* slot_edge,
                             double* out_xyz, int* out_tri, int* parent1, int* parent2, double* out_ind,
                             unsigned int* missing, cudaStream_t s);

// ---- manifold checks of the ForceManifold loop, input boundary edges (manifold.cu) ----
// fill = false: per-vertex incidence counts of the dual triangles; fill = true: the
// incidence lists at the scanned offsets (order within a list unspecified)
cudaError_t launch_dual_incidence(const int* dt, int64_t t, unsigned* cnt, const unsigned* off, unsigned* cursor,
                                  int* list, bool fill, cudaStream_t s);
// bad[k]: output vertex not manifold; has_nm[k]: holds a non-manifold input vertex
// (evaluated for the bad clusters only); issue[k]; unf[k]: neighbour of an issue
// cluster.  has_nm and unf must be zeroed by the caller.
cudaError_t launch_manifold_checks(const int* dt, const unsigned* off, const int* list, int k, const int* edge_int,
                                   int64_t ne, const int* label, int64_t n, const int* orig, const uint32_t* vf_row,
                                   const uint32_t* vf_face, const int* tri, const int* row, const int* size,
                                   unsigned char* bad, unsigned char* has_nm, unsigned char* issue,
                                   unsigned char* unf, cudaStream_t s);
cudaError_t launch_boundary_edge_flags(const int* edge_v, int64_t ne, const uint32_t* vf_row, const uint32_t* vf_face,
                                       const int* tri, uint32_t* flag, cudaStream_t s);
// one input boundary edge as FixMeshBoundaries reads it (vertex ids, clusters, ring sizes, points)
struct BoundaryEdge {
    int edge;
    int v[2];
    int c[2];
    int deg[2];
    int pad;
    double p1[3];
    double p2[3];
};
cudaError_t launch_boundary_gather(const int* ids, int64_t nb, const int* edge_v, const int* label_ext, const int* inv,
                                   const int* row, const double* xyz, BoundaryEdge* out, cudaStream_t s);

// ---- adjoint (adjoint.cu) ----
// Work arrays and inputs of the fixed-clustering adjoint (FP64).
struct AdjState {
    int64_t nv, nf;
    int k;
    const double* x;      // 3 nv
    const double* rho;    // nv or null
    double grad;          // gradation g
    const int* tri;
    const int* label;
    const uint32_t* vf_row;
    const uint32_t* vf_face;
    double* fn;           // 3 nf unit normals
    double* flen;         // nf |cr|
    double* farea;        // nf
    double* va;           // nv dual areas
    double* vA;           // 6 nv quadrics
    double* vw;           // nv weights (clamped)
    unsigned char* vclamp;
    double* cl;           // per cluster: S(3) W A(6) b(3) | E | c(3) | GS(3) GW GA(6) Gb(3)
    double* corner;       // 9 nf corner gradients
    double* ek;           // k per-cluster energies
};

size_t adjoint_bytes(int64_t nv, int64_t nf, int k);
AdjState adjoint_state(void* base, int64_t nv, int64_t nf, int k);

}  // namespace acvd

// Host orchestration of the GPU clustering (the MinimizeEnergy() seam) and the
// C ABI declared in include/acvd_gpu.h.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/acvd_gpu.h"
#include "primitives.cuh"
#include "state.cuh"

using namespace acvd;

namespace {

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t resize(size_t m) {
        if (m <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(m, 1) * sizeof(T));
        if (e == cudaSuccess) n = m;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { release(); }
};

}  // namespace

struct acvd_ctx {
    acvd_opts opts;
    std::string err;
    cudaStream_t s = nullptr;
    bool ready_mesh = false, ready_metric = false, ready_labels = false;

    // mesh
    int64_t nV = 0, nF = 0, nE = 0;
    int max_deg = 0;
    DBuf<double> xyz;
    DBuf<int> tri, row, col, edge_v;
    DBuf<unsigned> adj;
    int ncolors = 0;
    std::vector<int64_t> color_off;
    DBuf<int> color_items, cand_dest, cand_list;
    // acvd_adjoint_on_stream: orders the context's stream after the caller's and back
    cudaEvent_t adj_ev_in = nullptr, adj_ev_out = nullptr;
    // split evaluation of large colour classes (screen pass + work list)
    DBuf<int> work;
    DBuf<unsigned> work_count;
    int64_t split_min = 0;
    bool has_work = false;
    // internal item order: colour classes contiguous (perm: item -> original
    // vertex id, inv: original vertex id -> item); faces and edges in item ids
    DBuf<int> perm, inv, tri_int, edge_int, label_orig;
    DBuf<int4> ring8;              // first 8 ring slots per item
    // curvature: faces of every edge, edge of every ring slot, per-vertex outputs
    DBuf<int2> curv_poly;
    DBuf<int> curv_slot;
    DBuf<double> curv_ind;
    DBuf<float> curv_dirs;
    DBuf<char> curv_faces;
    DBuf<unsigned char> bflag;     // per item: maybe on a cluster boundary
    DBuf<int4> tcache;             // per item: cached boundary screen
    // sweep classes: either the colour classes, or one class holding every item
    // (claims alone keep committed moves on disjoint clusters; colours are kept
    // for hole filling)
    bool sweep_by_color = true;
    DBuf<int> all_items;
    std::vector<int64_t> sweep_off;
    const int* sweep_items = nullptr;
    int nclasses = 0;
    DBuf<unsigned> cand_prio, cand_count;

    // batch of meshes packed in one CSR (vertex and cluster offsets per mesh)
    int nmesh = 0;
    std::vector<int64_t> h_voff, h_koff;
    DBuf<int64_t> v_off, k_off;

    // vertex -> faces (increasing face id), kept for the adjoint
    DBuf<uint32_t> vf_row, vf_face;
    DBuf<char> adj_work;

    // items
    int metric = -1;
    DBuf<float4> xw, qa, ta;
    DBuf<float2> qb, tb;

    // clusters
    int K = 0;
    DBuf<int> label, size, stamp, evald;
    DBuf<int> uf_parent;           // clean: union-find links
    DBuf<int> fill_list;           // hole filling: unassigned items per colour class
    DBuf<unsigned> fill_cnt;
    DBuf<int64_t> fill_off;
    int64_t fill_block_max = 65536;   // ACVD_FILL_BLOCK_MAX: longest lists the single-block fill takes
    int union_tries = 1 << 16;        // ACVD_UNION_TRIES: attempts per union-find link before the fallback
    DBuf<unsigned long long> claim;
    DBuf<SweepState> dsweep;
    // relaxed steps
    DBuf<long long> fx_delta;
    DBuf<float4> fx_pow;
    DBuf<int> out_cnt, in_done, out_done;
    bool use_relaxed = true;       // ACVD_RELAXED=0 turns relaxed steps off
    DBuf<df> acc;
    DBuf<float4> ev;
    DBuf<double> energy;
    DBuf<unsigned long long> counters;
    unsigned long long* h_raw = nullptr;      // pinned copy of the counter stripes
    int* h_color = nullptr;                    // pinned colours of the host colourings
    int64_t h_color_cap = 0;
    unsigned long long h_counters[kNumCounters] = {};   // stripes summed
    DBuf<RunFlags> dflags;
    RunFlags flags{1, 0, 3, 1e-3f};
    int level = 3;
    int unconstrained = 0;
    double gradation = 0.0;

    // work
    DBuf<uint32_t> wk_a, wk_b, wk_c, wk_d, wk_cnt, wk_off;
    DBuf<int> comp, csize, multi, wk_int;
    DBuf<unsigned long long> best;
    DBuf<double> dtmp;
    Scratch scratch;

    // sweep graph; one event pair per colour class brackets its evaluation kernel
    cudaGraphExec_t sweep_exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> ev_eval;
    bool timing_broken = false;    // event timing unavailable on this device / driver
    int match_rounds = 1;          // claim/commit rounds per colour step (ACVD_MATCH_ROUNDS, up to kRounds)
    int eval_blocks = 0;           // evaluation kernels' blocks per SM, 3..5 (ACVD_EVAL_BLOCKS; 0 = defaults)
    int eval_threads = 256;        // their threads per block: 256, or 128 (ACVD_EVAL_THREADS)
    int64_t sweep_kernels = 0;     // kernels in the sweep last enqueued
    int64_t loop_relaxed_kernels = 0, loop_exact_kernels = 0;   // kernels per sweep of the graph loop
    int64_t exact_kernels = 0, relaxed_kernels = 0;
    DBuf<int> label_init;          // the assignment given to acvd_set_labels (for acvd_rewind)
    DBuf<unsigned char> frozen;    // per cluster (K + 1): IsClusterFreezed; used when has_frozen
    bool has_frozen = false;
    std::vector<unsigned char> h_frozen;
    // fixed vertices (FixedClusters) and anchored QEM clusters (Cluster::AnchorItem), as
    // vertex ids; the device copies hold items and are rebuilt for every K
    std::vector<int> h_fixed, h_anchor;
    DBuf<int> fixed_item, anchor_item, anchor_ids;
    DBuf<double> anchor_xyz;
    bool has_anchor = false;

    // set-up work buffers, kept between calls: a repeated set-up (same or smaller
    // mesh) allocates nothing, and so does not synchronise the device in cudaFree
    struct SetupWork {
        DBuf<int> col_new;
        DBuf<double> ind, farea, fnorm, wd, varea, wsum;
        DBuf<float> pd;
        DBuf<uint32_t> k1, k2, v2;
        DBuf<float4> t4;
        DBuf<float2> t2;
        DBuf<unsigned> maxbits;
    } setup;

    // persistent sweep kernel: loop state, grid barrier, energy partials, class
    // offsets, per-sweep log; grid = SMs x co-resident blocks (0: not available)
    DBuf<LoopState> dls;
    DBuf<GridBar> dbar;
    DBuf<double> esum;
    DBuf<long long> doff;
    DBuf<SweepLog> slog;
    int run_grid = -1;
    int run_grid_metric = -1;

    DevState state() {
        DevState st;
        st.n = nV;
        st.k = K;
        st.row = row.p;
        st.col = col.p;
        st.adj = adj.p;
        st.xw = xw.p;
        st.qa = qa.p;
        st.qb = qb.p;
        st.ta = ta.p;
        st.tb = tb.p;
        st.label = label.p;
        st.size = size.p;
        st.claim = claim.p;
        st.acc = acc.p;
        st.ev = ev.p;
        st.energy = energy.p;
        st.counters = counters.p;
        st.flags = dflags.p;
        st.sweep = dsweep.p;
        st.stamp = stamp.p;
        st.evald = evald.p;
        st.cand_list = cand_list.p;
        st.cand_count = cand_count.p;
        st.fx_delta = fx_delta.p;
        st.fx_pow = fx_pow.p;
        st.out_cnt = out_cnt.p;
        st.in_done = in_done.p;
        st.out_done = out_done.p;
        st.ring8 = ring8.p;
        st.bflag = bflag.p;
        st.tcache = tcache.p;
        st.orig = perm.p;
        st.inv = inv.p;
        st.frozen = has_frozen ? frozen.p : nullptr;
        st.anchor = has_anchor ? anchor_item.p : nullptr;
        st.anchor_xyz = has_anchor ? anchor_xyz.p : nullptr;
        st.nfixed = (int)h_fixed.size();
        st.fixed = h_fixed.empty() ? nullptr : fixed_item.p;
        st.work = has_work ? work.p : nullptr;
        st.work_count = has_work ? work_count.p : nullptr;
        return st;
    }
    cudaGraphExec_t relaxed_exec = nullptr;
    cudaGraphExec_t loop_exec = nullptr;   // device-side sweep loop (WHILE around relaxed / exact sweep)
    DBuf<double> loop_energy;              // energy after the loop's last relaxed sweep
    Scratch loop_scratch;                  // the loop graph's own summation scratch (never shared,
                                           // so no other call can move it under the graph)
    void drop_graph() {
        if (sweep_exec) cudaGraphExecDestroy(sweep_exec);
        sweep_exec = nullptr;
        if (relaxed_exec) cudaGraphExecDestroy(relaxed_exec);
        relaxed_exec = nullptr;
        if (loop_exec) cudaGraphExecDestroy(loop_exec);
        loop_exec = nullptr;
    }
    void drop_events() {
        for (cudaEvent_t e : ev_eval) cudaEventDestroy(e);
        ev_eval.clear();
    }
};

#define CK(call)                                                              \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return fail_cuda(ctx, _e, #call, __LINE__);   \
    } while (0)

static int fail(acvd_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

static int fail_cuda(acvd_ctx* ctx, cudaError_t e, const char* what, int line) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "CUDA error %d (%s) at engine.cu:%d: %s", (int)e, cudaGetErrorString(e), line,
                  what);
    return fail(ctx, ACVD_ERR_CUDA, buf);
}

static int sync_counters(acvd_ctx* ctx) {
    CK(cudaMemcpyAsync(ctx->h_raw, ctx->counters.p, kCounterWords * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    for (int c = 0; c < kNumCounters; c++) {
        unsigned long long v = 0;
        for (int q = 0; q < kStripes; q++) v += ctx->h_raw[q * kNumCounters + c];
        ctx->h_counters[c] = v;
    }
    return ACVD_OK;
}

// (a copy from pageable host memory returns once the source is staged, so neither this
// nor set_sweep_state waits for the stream)
static int upload_flags(acvd_ctx* ctx) {
    CK(cudaMemcpyAsync(ctx->dflags.p, &ctx->flags, sizeof(RunFlags), cudaMemcpyHostToDevice, ctx->s));
    return ACVD_OK;
}

// sweep counter and invalidation floor (every cluster counts as modified after `floor`)
// Also marks every item as maybe on a boundary: it is called whenever the labels
// changed wholesale (start, clean / fill at a convergence).
static int set_sweep_state(acvd_ctx* ctx, int sweep, int floor) {
    SweepState h{sweep, floor};
    CK(cudaMemcpyAsync(ctx->dsweep.p, &h, sizeof h, cudaMemcpyHostToDevice, ctx->s));
    CK(ctx->bflag.resize(ctx->nV));
    CK(ctx->tcache.resize(ctx->nV));
    CK(cudaMemsetAsync(ctx->bflag.p, 1, ctx->nV, ctx->s));
    return ACVD_OK;
}

// every stripe of one counter
static cudaError_t zero_counter(acvd_ctx* ctx, int which) {
    return cudaMemset2DAsync(ctx->counters.p + which, kNumCounters * sizeof(unsigned long long), 0,
                             sizeof(unsigned long long), kStripes, ctx->s);
}

// ---------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------
// Colour classes from this size on run the split evaluation: about four waves of
// the fused evaluation kernel's blocks on a 152-SM GB300.  Smaller classes (the
// 1024 x 512 torus has about 120,000 items per class) are latency-bound, and a
// second kernel per colour step would cost more than it saves.
constexpr int64_t kDefaultSplitMin = 600000;

// Greedy colouring in vertex order on the host: each vertex takes the smallest
// colour unused by its lower-numbered neighbours.  On meshes stored in a spatially
// coherent order (grids, scans) it gives 4 balanced classes where the device's
// hashed Jones-Plassmann colouring gives 6-7 with a few tiny ones.  Writes color[0..n)
// (the context's pinned buffer: a byte-colour, branch-free form of the loop measured
// slower inside the engine on a Grace core) and returns the largest colour, or -1
// when a vertex would need a 65th colour.
static int greedy_colors_host(const int32_t* row, const int32_t* col, int64_t n, int* color) {
    std::fill(color, color + n, -1);
    int maxc = 0;
    for (int64_t v = 0; v < n; v++) {
        unsigned long long used = 0ull;
        for (int p = row[v]; p < row[v + 1]; p++) {
            const int c = color[col[p]];
            if (c >= 0) used |= 1ull << c;
        }
        if (used == ~0ull) return -1;
        const int c = __builtin_ctzll(~used);
        color[v] = c;
        maxc = std::max(maxc, c);
    }
    return maxc;
}

// Empties the highest colour class where it can: each of its items takes a free
// colour below it, or swaps with its only neighbour u of some colour a when u can
// take another free colour below the top (u -> b, item -> a).  Sequential in item
// order, so deterministic; each pass visits only the items of the class it empties
// (listed in item order by one scan), since recolouring touches no other item of
// that class.  Returns the new largest colour.
static int squeeze_top_color(const int32_t* row, const int32_t* col, int* color, int64_t n, int maxc) {
    std::vector<int> top_items;
    while (maxc > 0) {
        const int top = maxc;
        top_items.clear();
        for (int64_t v = 0; v < n; v++)
            if (color[v] == top) top_items.push_back((int)v);
        bool emptied = true;
        for (const int v : top_items) {
            unsigned long long used = 0ull;
            for (int p = row[v]; p < row[v + 1]; p++) used |= 1ull << color[col[p]];
            const unsigned long long below = (1ull << top) - 1ull;
            if (~used & below) {
                color[v] = __builtin_ctzll(~used & below);
                continue;
            }
            bool done = false;
            for (int a = 0; a < top && !done; a++) {
                int u = -1, cnt = 0;
                for (int p = row[v]; p < row[v + 1]; p++)
                    if (color[col[p]] == a) { u = col[p]; cnt++; }
                if (cnt != 1) continue;
                unsigned long long uu = 1ull << a;
                for (int p = row[u]; p < row[u + 1]; p++) uu |= 1ull << color[col[p]];
                if (~uu & below) {
                    color[u] = __builtin_ctzll(~uu & below);
                    color[v] = a;
                    done = true;
                }
            }
            if (!done) emptied = false;
        }
        if (!emptied) break;
        maxc = top - 1;
    }
    return maxc;
}

// The context's pinned host array of n colours, through which the host colourings
// reach the device.
static int host_color_buffer(acvd_ctx* ctx, int64_t n, int** out) {
    if (ctx->h_color_cap < n) {
        if (ctx->h_color) cudaFreeHost(ctx->h_color);
        ctx->h_color = nullptr;
        ctx->h_color_cap = 0;
        CK(cudaMallocHost((void**)&ctx->h_color, n * sizeof(int)));
        ctx->h_color_cap = n;
    }
    *out = ctx->h_color;
    return ACVD_OK;
}

static int setup_colors(acvd_ctx* ctx, const int32_t* h_row, const int32_t* h_col) {
    const int64_t n = ctx->nV;
    CK(ctx->wk_int.resize(n));
    CK(cudaMemsetAsync(ctx->wk_int.p, 0xff, n * sizeof(int), ctx->s));   // color = -1
    CK(ctx->dtmp.resize(2));
    int* d_maxc = (int*)ctx->dtmp.p;
    CK(cudaMemsetAsync(d_maxc, 0, sizeof(int), ctx->s));
    // ACVD_COLORING=order: the host greedy colouring in vertex order instead (the
    // greedy loop is one serial chain through the previous vertex's colour; it runs
    // while the device sorts the vertex -> face incidences)
    const char* how = std::getenv("ACVD_COLORING");
    int maxc = 0;
    if (how && std::strcmp(how, "order") == 0) {
        int* hc = nullptr;
        int r = host_color_buffer(ctx, n, &hc);
        if (r) return r;
        maxc = greedy_colors_host(h_row, h_col, n, hc);
        if (maxc < 0) return fail(ctx, ACVD_ERR_UNSUPPORTED, "more than 64 colours needed (vertex valence too high)");
        CK(cudaMemcpyAsync(ctx->wk_int.p, hc, n * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    } else {
        // rounds in groups of four between host checks (a round after the last one
        // finds every item coloured and does nothing); the count left is the last
        // round's number of items still waiting for a neighbour
        int rounds = 0;
        for (;;) {
            for (int g = 0; g < 4; g++) {
                CK(zero_counter(ctx, kCntChanged));
                CK(launch_color_round(ctx->row.p, ctx->col.p, n, ctx->wk_int.p, ctx->counters.p + kCntChanged,
                                      d_maxc, ctx->s));
            }
            int r = sync_counters(ctx);
            if (r) return r;
            if (ctx->h_counters[kCntChanged] == 0) break;
            if ((rounds += 4) > 100000) return fail(ctx, ACVD_ERR_ITER_LIMIT, "graph colouring did not finish");
        }
        CK(cudaMemcpy(&maxc, d_maxc, sizeof(int), cudaMemcpyDeviceToHost));
        if (maxc >= 64) return fail(ctx, ACVD_ERR_UNSUPPORTED, "more than 64 colours needed (vertex valence too high)");
    }
    if (how && std::strcmp(how, "squeeze") == 0 && maxc > 0) {
        int* hc = nullptr;
        int r = host_color_buffer(ctx, n, &hc);
        if (r) return r;
        CK(cudaMemcpyAsync(hc, ctx->wk_int.p, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
        maxc = squeeze_top_color(h_row, h_col, hc, n, maxc);
        CK(cudaMemcpyAsync(ctx->wk_int.p, hc, n * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    ctx->ncolors = maxc + 1;
    // colour classes: stable sort of items by colour (items ascending inside a class)
    CK(ctx->wk_a.resize(n));
    CK(ctx->wk_b.resize(n));
    CK(ctx->wk_c.resize(n));
    CK(ctx->wk_d.resize(n));
    CK(cudaMemcpyAsync(ctx->wk_a.p, ctx->wk_int.p, n * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
    CK(ctx->color_items.resize(n));
    CK(launch_iota(n, (int*)ctx->wk_b.p, ctx->s));
    CK(radix_sort_pairs(ctx->wk_a.p, ctx->wk_b.p, ctx->wk_c.p, ctx->wk_d.p, n, 8, ctx->scratch, ctx->s));
    CK(cudaMemcpyAsync(ctx->color_items.p, ctx->wk_b.p, n * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
    CK(ctx->wk_cnt.resize(65));
    CK(launch_segment_offsets(ctx->wk_a.p, n, (uint32_t)ctx->ncolors, ctx->wk_cnt.p, ctx->s));
    std::vector<uint32_t> off(ctx->ncolors + 1);
    CK(cudaMemcpyAsync(off.data(), ctx->wk_cnt.p, off.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->color_off.assign(ctx->ncolors + 1, 0);
    int64_t mx = 0;
    for (int c = 0; c < ctx->ncolors; c++) {
        ctx->color_off[c + 1] = off[c + 1];
        mx = std::max<int64_t>(mx, (int64_t)off[c + 1] - off[c]);
    }
    // renumber: item t = the t-th entry of the colour-sorted list, so that every
    // colour class is the contiguous item range [color_off[c], color_off[c+1])
    CK(ctx->perm.resize(n));
    CK(ctx->inv.resize(n));
    CK(ctx->wk_a.resize(n + 1));
    CK(ctx->wk_b.resize(n + 1));
    CK(cudaMemcpyAsync(ctx->perm.p, ctx->color_items.p, n * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
    CK(launch_scatter_inv(ctx->perm.p, n, ctx->inv.p, ctx->s));
    {
        const int64_t ne2 = 2 * ctx->nE;
        DBuf<int>& col_new = ctx->setup.col_new;
        CK(col_new.resize(ne2));
        CK(launch_perm_degree(ctx->row.p, ctx->perm.p, n, ctx->wk_a.p, ctx->s));
        CK(exclusive_scan_u32(ctx->wk_a.p, ctx->wk_b.p, n + 1, nullptr, ctx->scratch, ctx->s));
        CK(launch_perm_ring(ctx->row.p, ctx->col.p, ctx->perm.p, ctx->inv.p, ctx->wk_b.p, n, col_new.p, ctx->s));
        CK(cudaMemcpyAsync(ctx->row.p, ctx->wk_b.p, (n + 1) * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
        CK(cudaMemcpyAsync(ctx->col.p, col_new.p, ne2 * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    CK(ctx->ring8.resize(2 * n));
    CK(launch_ring8(ctx->row.p, ctx->col.p, n, (int*)ctx->ring8.p, ctx->s));
    CK(ctx->tri_int.resize(3 * ctx->nF));
    CK(ctx->edge_int.resize(2 * ctx->nE));
    CK(launch_map_ids(ctx->tri.p, 3 * ctx->nF, ctx->inv.p, ctx->tri_int.p, ctx->s));
    CK(launch_map_ids(ctx->edge_v.p, 2 * ctx->nE, ctx->inv.p, ctx->edge_int.p, ctx->s));
    CK(ctx->all_items.resize(n));
    CK(launch_iota(n, ctx->all_items.p, ctx->s));
    CK(launch_iota(n, ctx->color_items.p, ctx->s));
    if (ctx->sweep_by_color) {
        ctx->sweep_off = ctx->color_off;
        ctx->sweep_items = ctx->color_items.p;
    } else {
        ctx->sweep_off = {0, n};
        ctx->sweep_items = ctx->all_items.p;
        mx = n;
    }
    ctx->nclasses = (int)ctx->sweep_off.size() - 1;
    CK(cudaStreamSynchronize(ctx->s));
    // classes of at least split_min items run the split evaluation (screen pass +
    // work list); ACVD_SPLIT_MIN overrides the threshold (0 = never split)
    {
        ctx->split_min = kDefaultSplitMin;
        if (const char* e = std::getenv("ACVD_SPLIT_MIN")) ctx->split_min = std::atoll(e);
        int64_t wmax = 0;
        for (int c = 0; c < ctx->nclasses; c++) {
            const int64_t cnt = ctx->sweep_off[c + 1] - ctx->sweep_off[c];
            if (ctx->split_min > 0 && cnt >= ctx->split_min)
                wmax = std::max<int64_t>(wmax, kWorkStripes * work_cap(cnt));
        }
        if (wmax > 0) {
            CK(ctx->work.resize(wmax));
            CK(ctx->work_count.resize(64 * kWorkStripes));
            CK(cudaMemsetAsync(ctx->work_count.p, 0, 64 * kWorkStripes * sizeof(unsigned), ctx->s));
        }
        ctx->has_work = wmax > 0;
    }
    CK(ctx->cand_dest.resize(mx));
    CK(ctx->cand_prio.resize(mx));
    CK(ctx->cand_list.resize(mx));
    CK(ctx->cand_count.resize(64));
    CK(ctx->evald.resize(n));
    CK(cudaMemsetAsync(ctx->cand_dest.p, 0xff, mx * sizeof(int), ctx->s));
    CK(cudaMemsetAsync(ctx->cand_count.p, 0, 64 * sizeof(unsigned), ctx->s));
    return ACVD_OK;
}

extern "C" {

void acvd_default_opts(acvd_opts* o) {
    o->device = 0;
    o->use_graphs = 1;
    o->max_loops = 5000000;
    o->max_convergences = 1000000000;
    o->kernel_timing = 0;
    o->persistent = 0;
}

acvd_ctx* acvd_create(const acvd_opts* opts) {
    acvd_ctx* ctx = new acvd_ctx;
    if (opts) ctx->opts = *opts;
    else acvd_default_opts(&ctx->opts);
    if (const char* c = std::getenv("ACVD_SWEEP_COLORS")) ctx->sweep_by_color = std::atoi(c) != 0;
    if (const char* c = std::getenv("ACVD_RELAXED")) ctx->use_relaxed = std::atoi(c) != 0;
    if (const char* b = std::getenv("ACVD_EVAL_BLOCKS")) ctx->eval_blocks = std::atoi(b);
    if (const char* u = std::getenv("ACVD_UNION_TRIES")) ctx->union_tries = std::max(0, std::atoi(u));
    if (const char* f = std::getenv("ACVD_FILL_BLOCK_MAX"))
        ctx->fill_block_max = std::max<int64_t>(0, std::min<int64_t>(std::atoll(f), 1ll << 30));
    if (const char* t = std::getenv("ACVD_EVAL_THREADS")) {
        const int v = std::atoi(t);
        ctx->eval_threads = v == 128 ? 128 : 256;
    }
    if (const char* r = std::getenv("ACVD_MATCH_ROUNDS")) {
        const int v = std::atoi(r);
        if (v >= 1 && v <= kRounds) ctx->match_rounds = v;
    }
    if (cudaSetDevice(ctx->opts.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->h_raw, kCounterWords * sizeof(unsigned long long)) != cudaSuccess ||
        ctx->counters.resize(kCounterWords) != cudaSuccess || ctx->dflags.resize(1) != cudaSuccess ||
        ctx->dsweep.resize(1) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return nullptr;
    }
    cudaMemset(ctx->counters.p, 0, kCounterWords * sizeof(unsigned long long));
    return ctx;
}

void acvd_destroy(acvd_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->opts.device);
    if (ctx->s) cudaStreamSynchronize(ctx->s);
    ctx->drop_graph();
    ctx->drop_events();
    if (ctx->h_raw) cudaFreeHost(ctx->h_raw);
    if (ctx->h_color) cudaFreeHost(ctx->h_color);
    if (ctx->adj_ev_in) cudaEventDestroy(ctx->adj_ev_in);
    if (ctx->adj_ev_out) cudaEventDestroy(ctx->adj_ev_out);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->s) cudaStreamDestroy(ctx->s);
    delete ctx;
}

const char* acvd_last_error(const acvd_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* acvd_stream(acvd_ctx* ctx) { return ctx ? (void*)ctx->s : nullptr; }

int acvd_set_mesh(acvd_ctx* ctx, int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri,
                  const int32_t* csr_row, const int32_t* csr_col, int64_t n_edges, const int32_t* edge_v) {
    if (!ctx) return ACVD_ERR_ARG;
    if (n_vertices <= 0 || n_faces <= 0 || n_edges <= 0 || !xyz || !tri || !csr_row || !csr_col || !edge_v)
        return fail(ctx, ACVD_ERR_ARG, "acvd_set_mesh: empty mesh or null array");
    if (n_vertices >= (1ll << 26)) return fail(ctx, ACVD_ERR_UNSUPPORTED, "more than 2^26 vertices");
    if (csr_row[0] != 0 || csr_row[n_vertices] != 2 * n_edges)
        return fail(ctx, ACVD_ERR_ARG, "acvd_set_mesh: ring CSR does not hold 2 * n_edges entries");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->drop_graph();
    ctx->ready_mesh = ctx->ready_metric = ctx->ready_labels = false;
    ctx->h_fixed.clear();    // vertex ids of the previous mesh
    ctx->h_anchor.clear();
    ctx->has_anchor = false;
    ctx->nmesh = 0;
    ctx->nV = n_vertices;
    ctx->nF = n_faces;
    ctx->nE = n_edges;
    CK(ctx->xyz.resize(3 * n_vertices));
    CK(ctx->tri.resize(3 * n_faces));
    CK(ctx->row.resize(n_vertices + 1));
    CK(ctx->col.resize(2 * n_edges));
    CK(ctx->edge_v.resize(2 * n_edges));
    CK(ctx->adj.resize(2 * n_edges));
    CK(cudaMemcpyAsync(ctx->xyz.p, xyz, 3 * n_vertices * sizeof(double), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(ctx->tri.p, tri, 3 * n_faces * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(ctx->row.p, csr_row, (n_vertices + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(ctx->col.p, csr_col, 2 * n_edges * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(ctx->edge_v.p, edge_v, 2 * n_edges * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    {
        // every id in range before any kernel indexes with it
        CK(ctx->dtmp.resize(2));
        unsigned* bad = (unsigned*)ctx->dtmp.p;
        unsigned h_bad = 0;
        CK(cudaMemsetAsync(bad, 0, sizeof(unsigned), ctx->s));
        CK(launch_validate_mesh(ctx->row.p, ctx->col.p, n_vertices, 2 * n_edges, ctx->tri.p, 3 * n_faces,
                                ctx->edge_v.p, 2 * n_edges, bad, ctx->s));
        CK(cudaMemcpyAsync(&h_bad, bad, sizeof h_bad, cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
        if (h_bad)
            return fail(ctx, ACVD_ERR_ARG, "acvd_set_mesh: " + std::to_string(h_bad) +
                                                " ring offsets decrease or vertex ids lie outside [0, n_vertices)");
    }
    // vertex -> faces in increasing face id (original ids): item build, curvature,
    // adjoint and post-placement read it
    {
        DBuf<uint32_t>&k1 = ctx->setup.k1, &k2 = ctx->setup.k2, &v2 = ctx->setup.v2;
        CK(k1.resize(3 * n_faces));
        CK(k2.resize(3 * n_faces));
        CK(v2.resize(3 * n_faces));
        CK(ctx->vf_row.resize(n_vertices + 1));
        CK(ctx->vf_face.resize(3 * n_faces));
        CK(launch_vertex_keys(ctx->tri.p, n_faces, k1.p, ctx->vf_face.p, ctx->s));
        CK(radix_sort_pairs(k1.p, ctx->vf_face.p, k2.p, v2.p, 3 * n_faces, bits_for((uint64_t)n_vertices),
                            ctx->scratch, ctx->s));
        CK(launch_segment_offsets(k1.p, 3 * n_faces, (uint32_t)n_vertices, ctx->vf_row.p, ctx->s));
    }
    // colouring on the input rings, then the items in internal order
    int r = setup_colors(ctx, csr_row, csr_col);
    if (r) return r;
    int* d_maxdeg = nullptr;
    CK(ctx->dtmp.resize(2));
    d_maxdeg = (int*)ctx->dtmp.p;
    CK(cudaMemsetAsync(d_maxdeg, 0, sizeof(int), ctx->s));
    CK(launch_ring_adjacency(ctx->row.p, ctx->col.p, n_vertices, ctx->adj.p, d_maxdeg, ctx->s));
    CK(cudaMemcpyAsync(&ctx->max_deg, d_maxdeg, sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->ready_mesh = true;
    return ACVD_OK;
}

int acvd_set_metric(acvd_ctx* ctx, int metric, const double* indicator, const float* principal_dirs,
                    double gradation) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh) return fail(ctx, ACVD_ERR_ARG, "acvd_set_metric before acvd_set_mesh");
    if (metric < 0 || metric > 2) return fail(ctx, ACVD_ERR_ARG, "unknown metric");
    const bool use_ind = metric == kAniso ? gradation != 0.0 : gradation > 0.0;
    if (use_ind && !indicator) return fail(ctx, ACVD_ERR_ARG, "gradation set but no indicator given");
    if (metric == kAniso && !principal_dirs)
        return fail(ctx, ACVD_ERR_ARG, "the quadric-anisotropic metric needs principal directions");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->drop_graph();
    ctx->metric = metric;
    const int64_t nv = ctx->nV, nf = ctx->nF;
    DBuf<double>&ind = ctx->setup.ind, &farea = ctx->setup.farea, &fnorm = ctx->setup.fnorm, &wd = ctx->setup.wd,
                &varea = ctx->setup.varea, &wsum = ctx->setup.wsum;
    DBuf<float>& pd = ctx->setup.pd;
    if (use_ind) {
        CK(ind.resize(nv));
        CK(cudaMemcpyAsync(ind.p, indicator, nv * sizeof(double), cudaMemcpyHostToDevice, ctx->s));
    }
    if (metric == kAniso) {
        CK(pd.resize(6 * nv));
        CK(cudaMemcpyAsync(pd.p, principal_dirs, 6 * nv * sizeof(float), cudaMemcpyHostToDevice, ctx->s));
    }
    CK(farea.resize(nf));
    CK(fnorm.resize(3 * nf));
    CK(wd.resize(nv));
    CK(varea.resize(nv));
    CK(wsum.resize(1));
    CK(launch_face_geometry(ctx->xyz.p, ctx->tri.p, nf, farea.p, fnorm.p, ctx->s));
    CK(ctx->xw.resize(nv));
    if (metric != kIso) {
        CK(ctx->qa.resize(nv));
        CK(ctx->qb.resize(nv));
    }
    if (metric == kAniso) {
        CK(ctx->ta.resize(nv));
        CK(ctx->tb.resize(nv));
    }
    CK(launch_vertex_items(metric, nv, ctx->xyz.p, ctx->vf_row.p, ctx->vf_face.p, farea.p, fnorm.p, use_ind ? ind.p : nullptr,
                           gradation, wd.p, varea.p, ctx->qa.p, ctx->qb.p, ctx->s));
    ctx->gradation = gradation;
    const double ratio = metric == kQEM ? 10000.0 : 100000.0;
    if (ctx->nmesh > 0) {
        CK(wsum.resize(ctx->nmesh));
        CK(launch_mesh_sums(wd.p, ctx->v_off.p, ctx->nmesh, wsum.p, ctx->s));
        CK(launch_finish_items(metric, nv, ctx->xyz.p, wd.p, varea.p, wsum.p, ctx->v_off.p, ctx->nmesh, ratio, pd.p,
                               ctx->xw.p, ctx->ta.p, ctx->tb.p, ctx->s));
    } else {
        CK(sum_f64(wd.p, nv, wsum.p, ctx->scratch, ctx->s));
        CK(launch_finish_items(metric, nv, ctx->xyz.p, wd.p, varea.p, wsum.p, nullptr, 0, ratio, pd.p, ctx->xw.p,
                               ctx->ta.p, ctx->tb.p, ctx->s));
    }
    // item records into internal order
    {
        DBuf<float4>& t4 = ctx->setup.t4;
        DBuf<float2>& t2 = ctx->setup.t2;
        CK(t4.resize(nv));
        CK(launch_gather_f4(ctx->xw.p, ctx->perm.p, nv, t4.p, ctx->s));
        CK(cudaMemcpyAsync(ctx->xw.p, t4.p, nv * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->s));
        if (metric != kIso) {
            CK(t2.resize(nv));
            CK(launch_gather_f4(ctx->qa.p, ctx->perm.p, nv, t4.p, ctx->s));
            CK(cudaMemcpyAsync(ctx->qa.p, t4.p, nv * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->s));
            CK(launch_gather_f2(ctx->qb.p, ctx->perm.p, nv, t2.p, ctx->s));
            CK(cudaMemcpyAsync(ctx->qb.p, t2.p, nv * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->s));
        }
        if (metric == kAniso) {
            CK(launch_gather_f4(ctx->ta.p, ctx->perm.p, nv, t4.p, ctx->s));
            CK(cudaMemcpyAsync(ctx->ta.p, t4.p, nv * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->s));
            CK(launch_gather_f2(ctx->tb.p, ctx->perm.p, nv, t2.p, ctx->s));
            CK(cudaMemcpyAsync(ctx->tb.p, t2.p, nv * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->s));
        }
        CK(cudaStreamSynchronize(ctx->s));
    }
    // fixed-point scales of the relaxed steps: any sum of up to N contributions of
    // component j stays below 2^62 units
    {
        DBuf<unsigned>& maxbits = ctx->setup.maxbits;
        CK(maxbits.resize(32));
        CK(cudaMemsetAsync(maxbits.p, 0, 32 * sizeof(unsigned), ctx->s));
        DevState st = ctx->state();
        CK(launch_fx_scale(metric, st, maxbits.p, ctx->s));
        unsigned hb[32];
        CK(cudaMemcpyAsync(hb, maxbits.p, sizeof hb, cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
        // the largest power of two 2^e with N * max|contribution| * 2^e < 2^62 (hi part
        // bound, with a margin for the lo parts), split into two factors 2^e1 2^e2
        float4 sc[32];
        for (int q = 0; q < 32; q++) {
            float mx;
            std::memcpy(&mx, &hb[q], sizeof mx);
            int e = 0;
            if (mx > 0.f) e = (int)std::floor(62.0 - std::log2((double)nv * (double)mx * 1.0001));
            const int e1 = e / 2, e2 = e - e1;
            sc[q] = make_float4(std::ldexp(1.0f, e1), std::ldexp(1.0f, e2), std::ldexp(1.0f, -e1),
                                std::ldexp(1.0f, -e2));
        }
        CK(ctx->fx_pow.resize(32));
        CK(cudaMemcpyAsync(ctx->fx_pow.p, sc, sizeof sc, cudaMemcpyHostToDevice, ctx->s));
    }
    CK(cudaStreamSynchronize(ctx->s));
    ctx->ready_metric = true;
    return ACVD_OK;
}

int acvd_set_batch(acvd_ctx* ctx, int n_mesh, const int64_t* vertex_offsets, const int32_t* cluster_offsets) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh) return fail(ctx, ACVD_ERR_ARG, "acvd_set_batch before acvd_set_mesh");
    if (n_mesh < 0 || (n_mesh > 0 && (!vertex_offsets || !cluster_offsets)))
        return fail(ctx, ACVD_ERR_ARG, "acvd_set_batch: bad offsets");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->drop_graph();
    ctx->ready_metric = ctx->ready_labels = false;
    ctx->nmesh = n_mesh;
    ctx->h_voff.assign(vertex_offsets, vertex_offsets + (n_mesh ? n_mesh + 1 : 0));
    ctx->h_koff.clear();
    for (int m = 0; m <= n_mesh && n_mesh > 0; m++) ctx->h_koff.push_back(cluster_offsets[m]);
    if (n_mesh == 0) return ACVD_OK;
    if (ctx->h_voff[0] != 0 || ctx->h_voff[n_mesh] != ctx->nV)
        return fail(ctx, ACVD_ERR_ARG, "acvd_set_batch: vertex offsets must run from 0 to n_vertices");
    for (int m = 0; m < n_mesh; m++)
        if (ctx->h_voff[m + 1] <= ctx->h_voff[m] || ctx->h_koff[m + 1] <= ctx->h_koff[m] || ctx->h_koff[0] != 0)
            return fail(ctx, ACVD_ERR_ARG, "acvd_set_batch: offsets must increase from 0");
    CK(ctx->v_off.resize(n_mesh + 1));
    CK(ctx->k_off.resize(n_mesh + 1));
    CK(cudaMemcpyAsync(ctx->v_off.p, ctx->h_voff.data(), (n_mesh + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->s));
    CK(cudaMemcpyAsync(ctx->k_off.p, ctx->h_koff.data(), (n_mesh + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

int acvd_set_quadrics_optimization_level(acvd_ctx* ctx, int level) {
    if (!ctx || level < 0 || level > 3) return fail(ctx, ACVD_ERR_ARG, "level must be 0..3");
    ctx->level = level;
    return ACVD_OK;
}

int acvd_set_unconstrained_initialization(acvd_ctx* ctx, int on) {
    if (!ctx) return ACVD_ERR_ARG;
    ctx->unconstrained = on ? 1 : 0;
    return ACVD_OK;
}

static int sync_fixed(acvd_ctx* ctx);

int acvd_set_labels(acvd_ctx* ctx, int32_t k, const int32_t* labels) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh) return fail(ctx, ACVD_ERR_ARG, "acvd_set_labels before acvd_set_mesh");
    if (k <= 0 || !labels) return fail(ctx, ACVD_ERR_ARG, "acvd_set_labels: K must be positive");
    if (k >= (1 << 21)) return fail(ctx, ACVD_ERR_UNSUPPORTED, "more than 2^21 clusters");
    CK(cudaSetDevice(ctx->opts.device));
    if (ctx->K != k || ctx->has_frozen) ctx->drop_graph();
    ctx->has_frozen = false;   // a new clustering starts with no frozen cluster
    ctx->K = k;
    const int ms = ctx->metric >= 0 ? ctx->metric : kAniso;
    CK(ctx->label.resize(ctx->nV));
    CK(ctx->size.resize(k + 1));
    CK(ctx->stamp.resize(k + 1));
    CK(ctx->fx_delta.resize((size_t)(k + 1) * acc_stride(kAniso)));
    CK(ctx->out_cnt.resize(k + 1));
    CK(ctx->in_done.resize(k + 1));
    CK(ctx->out_done.resize(k + 1));
    CK(ctx->claim.resize(k + 1));
    CK(ctx->acc.resize((size_t)(k + 1) * acc_stride(kAniso)));
    CK(ctx->ev.resize((size_t)(k + 1) * ev_stride(kAniso)));
    CK(ctx->energy.resize(k + 1));
    (void)ms;
    CK(ctx->label_init.resize(ctx->nV));
    CK(ctx->label_orig.resize(ctx->nV));
    CK(cudaMemcpyAsync(ctx->label_orig.p, labels, ctx->nV * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    // the range check runs in the gather: a label outside [0, K] fails the call
    CK(ctx->dtmp.resize(2));
    unsigned* bad = (unsigned*)ctx->dtmp.p;
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned), ctx->s));
    CK(launch_gather_labels(ctx->label_orig.p, ctx->perm.p, ctx->nV, k, ctx->label.p, bad, ctx->s));
    CK(cudaMemcpyAsync(ctx->label_init.p, ctx->label.p, ctx->nV * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
    unsigned h_bad = 0;
    CK(cudaMemcpyAsync(&h_bad, bad, sizeof h_bad, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (h_bad) {
        ctx->ready_labels = false;
        return fail(ctx, ACVD_ERR_ARG, std::to_string(h_bad) + " labels outside [0, K]");
    }
    ctx->ready_labels = true;
    if (!ctx->h_fixed.empty() || ctx->has_anchor || !ctx->h_anchor.empty()) return sync_fixed(ctx);
    return ACVD_OK;
}

// Device copies of the fixed items and the anchored clusters for the current K
// (clusters added since the anchors were given have none).
static int sync_fixed(acvd_ctx* ctx) {
    const int nf = (int)ctx->h_fixed.size(), K = ctx->K;
    if (nf > K) return fail(ctx, ACVD_ERR_ARG, std::to_string(nf) + " fixed vertices for " + std::to_string(K) +
                                                   " clusters");
    std::vector<int> ids(ctx->h_fixed);
    bool any = false;
    for (int c = 0; c < K; c++) {
        const int a = c < (int)ctx->h_anchor.size() ? ctx->h_anchor[c] : -1;
        ids.push_back(a);
        any |= a >= 0;
    }
    ctx->drop_graph();   // the captured sweeps hold the state's pointers
    CK(ctx->anchor_ids.resize(nf + K));
    CK(cudaMemcpyAsync(ctx->anchor_ids.p, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    if (nf > 0) {
        CK(ctx->fixed_item.resize(nf));
        CK(launch_anchor_setup(ctx->anchor_ids.p, nf, ctx->inv.p, ctx->xyz.p, ctx->fixed_item.p, nullptr, ctx->s));
    }
    ctx->has_anchor = any;
    if (any) {
        CK(ctx->anchor_item.resize(K));
        CK(ctx->anchor_xyz.resize(3 * (size_t)K));
        CK(launch_anchor_setup(ctx->anchor_ids.p + nf, K, ctx->inv.p, ctx->xyz.p, ctx->anchor_item.p,
                               ctx->anchor_xyz.p, ctx->s));
    }
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

int acvd_set_fixed_clusters(acvd_ctx* ctx, int32_t n_fixed, const int32_t* vertex_ids) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh) return fail(ctx, ACVD_ERR_ARG, "acvd_set_fixed_clusters before acvd_set_mesh");
    if (n_fixed < 0 || (n_fixed > 0 && !vertex_ids)) return fail(ctx, ACVD_ERR_ARG, "acvd_set_fixed_clusters: bad list");
    for (int c = 0; c < n_fixed; c++)
        if (vertex_ids[c] < 0 || vertex_ids[c] >= ctx->nV)
            return fail(ctx, ACVD_ERR_ARG, "acvd_set_fixed_clusters: vertex id outside [0, n_vertices)");
    if (ctx->ready_labels && n_fixed > ctx->K)
        return fail(ctx, ACVD_ERR_ARG, "acvd_set_fixed_clusters: more fixed vertices than clusters");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->h_fixed.assign(vertex_ids, vertex_ids + n_fixed);
    return ctx->ready_labels ? sync_fixed(ctx) : ACVD_OK;
}

int acvd_set_anchor_items(acvd_ctx* ctx, int32_t n, const int32_t* anchors) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_metric) return fail(ctx, ACVD_ERR_ARG, "acvd_set_anchor_items before acvd_set_metric");
    if (ctx->metric != kQEM && n > 0)
        return fail(ctx, ACVD_ERR_UNSUPPORTED, "anchor items belong to the QEM metric's clusters");
    if (n < 0 || (n > 0 && !anchors)) return fail(ctx, ACVD_ERR_ARG, "acvd_set_anchor_items: bad list");
    for (int c = 0; c < n; c++)
        if (anchors[c] < -1 || anchors[c] >= ctx->nV)
            return fail(ctx, ACVD_ERR_ARG, "acvd_set_anchor_items: vertex id outside [-1, n_vertices)");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->h_anchor.assign(anchors, anchors + n);
    return ctx->ready_labels ? sync_fixed(ctx) : ACVD_OK;
}

int acvd_set_frozen_clusters(acvd_ctx* ctx, const uint8_t* frozen) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_set_frozen_clusters before acvd_set_labels");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->drop_graph();   // the captured sweeps hold the state's pointers
    if (!frozen) {
        ctx->has_frozen = false;
        return ACVD_OK;
    }
    ctx->h_frozen.assign(frozen, frozen + ctx->K);
    for (auto& f : ctx->h_frozen) f = f ? 1 : 0;
    ctx->h_frozen.push_back(0);   // the null label K is never frozen
    CK(ctx->frozen.resize(ctx->K + 1));
    CK(cudaMemcpyAsync(ctx->frozen.p, ctx->h_frozen.data(), ctx->K + 1, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    ctx->has_frozen = true;
    return ACVD_OK;
}

int acvd_get_frozen_clusters(acvd_ctx* ctx, uint8_t* frozen) {
    if (!ctx || !frozen) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_get_frozen_clusters before acvd_set_labels");
    for (int c = 0; c < ctx->K; c++) frozen[c] = ctx->has_frozen ? ctx->h_frozen[c] : 0;
    return ACVD_OK;
}

int acvd_rewind(acvd_ctx* ctx) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_rewind before acvd_set_labels");
    CK(cudaSetDevice(ctx->opts.device));
    CK(cudaMemcpyAsync(ctx->label.p, ctx->label_init.p, ctx->nV * sizeof(int), cudaMemcpyDeviceToDevice, ctx->s));
    return ACVD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// MinimizeEnergy building blocks
// ---------------------------------------------------------------------------
static int recompute(acvd_ctx* ctx) {
    DevState st = ctx->state();
    const int64_t n = ctx->nV;
    const int K = ctx->K;
    CK(ctx->wk_a.resize(n));
    CK(ctx->wk_b.resize(n));
    CK(ctx->wk_c.resize(n));
    CK(ctx->wk_d.resize(n));
    CK(ctx->wk_cnt.resize(K + 1));
    CK(ctx->wk_off.resize(K + 1));
    CK(cudaMemsetAsync(ctx->wk_cnt.p, 0, (K + 1) * sizeof(uint32_t), ctx->s));
    CK(launch_cluster_keys(st, ctx->wk_a.p, ctx->wk_b.p, ctx->wk_cnt.p, ctx->s));
    CK(radix_sort_pairs(ctx->wk_a.p, ctx->wk_b.p, ctx->wk_c.p, ctx->wk_d.p, n, bits_for((uint64_t)K), ctx->scratch,
                        ctx->s));
    CK(exclusive_scan_u32(ctx->wk_cnt.p, ctx->wk_off.p, K + 1, nullptr, ctx->scratch, ctx->s));
    CK(launch_reduce_clusters(ctx->metric, st, ctx->wk_b.p, ctx->wk_off.p, ctx->wk_cnt.p, ctx->s));
    CK(launch_update_all(ctx->metric, st, ctx->s));
    return ACVD_OK;
}

// FillHolesInClustering (Common/vtkUniformClustering.h:552-633): rounds of the colour
// classes in order until no unassigned item can join a cluster.  The rounds run over
// lists of the unassigned items, collected once: up to fill_block_max of them (65,536;
// ACVD_FILL_BLOCK_MAX), every round in one single-block launch; more, one launch per
// class and round with a host check per round.  Both give the same labels.
// *unassigned: the items left (collected minus filled).

static int fill_holes(acvd_ctx* ctx, int* unassigned) {
    DevState st = ctx->state();
    const int nc = ctx->ncolors;
    CK(ctx->fill_list.resize(ctx->nV));
    CK(ctx->fill_cnt.resize(nc + 1));   // [nc]: the single-block pass's error flag
    CK(ctx->fill_off.resize(nc + 1));
    CK(cudaMemsetAsync(ctx->fill_cnt.p, 0, (nc + 1) * sizeof(unsigned), ctx->s));
    CK(cudaMemcpyAsync(ctx->fill_off.p, ctx->color_off.data(), (nc + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->s));
    CK(launch_fill_collect(st, ctx->fill_off.p, nc, ctx->fill_list.p, ctx->fill_cnt.p, ctx->s));
    // the single-block pass, which declines lists longer than fill_block_max; the
    // counts and its status come back with one host round trip
    CK(zero_counter(ctx, kCntAssigned));
    CK(launch_fill_block(st, ctx->fill_list.p, ctx->fill_off.p, nc, ctx->fill_cnt.p, ctx->fill_cnt.p + nc,
                         (unsigned)ctx->fill_block_max, ctx->s));
    std::vector<unsigned> cnt(nc + 1);
    CK(cudaMemcpyAsync(cnt.data(), ctx->fill_cnt.p, (nc + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->s));
    {
        int r = sync_counters(ctx);
        if (r) return r;
    }
    int64_t total = 0;
    for (int c = 0; c < nc; c++) total += cnt[c];
    const unsigned status = cnt[nc];
    int64_t filled = 0;
    if (status == 1) return fail(ctx, ACVD_ERR_ITER_LIMIT, "hole filling did not finish");
    if (status == 0) {
        filled = (int64_t)ctx->h_counters[kCntAssigned];
    } else {
        for (int round = 0;; round++) {
            if (round > 1000000) return fail(ctx, ACVD_ERR_ITER_LIMIT, "hole filling did not finish");
            CK(zero_counter(ctx, kCntAssigned));
            for (int c = 0; c < nc; c++)
                if (cnt[c])
                    CK(launch_fill_list(st, ctx->fill_list.p + ctx->color_off[c], ctx->fill_cnt.p + c, cnt[c],
                                        ctx->s));
            int r = sync_counters(ctx);
            if (r) return r;
            if (ctx->h_counters[kCntAssigned] == 0) break;
            filled += (int64_t)ctx->h_counters[kCntAssigned];
        }
    }
    if (unassigned) *unassigned = (int)(total - filled);
    return ACVD_OK;
}

static int clean(acvd_ctx* ctx, int* n_disconnected) {
    DevState st = ctx->state();
    const int64_t n = ctx->nV;
    CK(ctx->comp.resize(n));
    CK(ctx->csize.resize(n));
    CK(ctx->multi.resize(ctx->K + 1));
    CK(ctx->best.resize(ctx->K + 1));
    // union-find in one pass; should a link give up (after union_tries attempts, a bound
    // never met in practice at the default), min-id propagation with pointer jumping
    // gives the same components
    CK(ctx->uf_parent.resize(n));
    CK(zero_counter(ctx, kCntChanged));
    CK(launch_comp_union(st, ctx->comp.p, ctx->uf_parent.p, ctx->union_tries, ctx->s));
    {
        int r = sync_counters(ctx);
        if (r) return r;
    }
    if (ctx->h_counters[kCntChanged] != 0) {
        CK(launch_comp_init(st, ctx->comp.p, ctx->s));
        for (int it = 0;; it++) {
            if (it > 100000) return fail(ctx, ACVD_ERR_ITER_LIMIT, "connected-component labelling did not converge");
            CK(zero_counter(ctx, kCntChanged));
            // several propagation steps between host checks
            for (int j = 0; j < 4; j++) CK(launch_comp_step(st, ctx->comp.p, ctx->s));
            int r = sync_counters(ctx);
            if (r) return r;
            if (ctx->h_counters[kCntChanged] == 0) break;
        }
    }
    CK(cudaMemsetAsync(ctx->csize.p, 0, n * sizeof(int), ctx->s));
    CK(cudaMemsetAsync(ctx->best.p, 0, (ctx->K + 1) * sizeof(unsigned long long), ctx->s));
    CK(cudaMemsetAsync(ctx->multi.p, 0, (ctx->K + 1) * sizeof(int), ctx->s));
    CK(zero_counter(ctx, kCntDisconnected));
    CK(launch_comp_finish(st, ctx->comp.p, ctx->csize.p, ctx->best.p, ctx->multi.p, ctx->s));
    int r = sync_counters(ctx);
    if (r) return r;
    *n_disconnected = (int)ctx->h_counters[kCntDisconnected];
    return ACVD_OK;
}

extern "C" int acvd_clean_clustering(acvd_ctx* ctx, int32_t* n_disconnected) {
    if (!ctx || !n_disconnected) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_clean_clustering before acvd_set_labels");
    CK(cudaSetDevice(ctx->opts.device));
    int n = 0;
    const int r = clean(ctx, &n);
    if (r) return r;
    *n_disconnected = n;
    return ACVD_OK;
}

// one sweep: every colour class once (eval + apply per class).  With kernel
// timing on, an event pair per colour brackets the evaluation kernel; the pairs
// are recorded inside the captured graph and read after the sweep's sync.
static int enqueue_sweep(acvd_ctx* ctx, bool timing, bool relaxed) {
    DevState st = ctx->state();
    CK(launch_begin_sweep(st, ctx->nclasses, !relaxed, ctx->s));   // exact sweeps: claims reset once
    int64_t kernels = 1;
    for (int c = 0; c < ctx->nclasses; c++) {
        const int item0 = (int)ctx->sweep_off[c];   // classes are contiguous item ranges
        const int64_t cnt = ctx->sweep_off[c + 1] - ctx->sweep_off[c];
        if (cnt == 0) continue;
        // cudaEventRecordExternal makes the records real graph nodes when captured
        if (timing) CK(cudaEventRecordWithFlags(ctx->ev_eval[2 * c], ctx->s, cudaEventRecordExternal));
        const bool split = ctx->has_work && ctx->split_min > 0 && cnt >= ctx->split_min;
        CK(launch_eval(ctx->metric, st, item0, cnt, c, ctx->cand_dest.p, ctx->cand_prio.p, !relaxed, split,
                       ctx->eval_blocks, ctx->eval_threads, ctx->s));
        if (split) kernels++;
        if (timing) CK(cudaEventRecordWithFlags(ctx->ev_eval[2 * c + 1], ctx->s, cudaEventRecordExternal));
        if (relaxed) {
            CK(launch_relaxed_step(ctx->metric, st, item0, cnt, c, ctx->cand_dest.p, ctx->s));
            kernels += 3;
            continue;
        }
        CK(launch_apply(ctx->metric, st, item0, cnt, c, 0, ctx->cand_dest.p, ctx->cand_prio.p, ctx->s));
        kernels += 2;
        for (int r = 1; r < ctx->match_rounds; r++) {
            CK(launch_reclaim(st, item0, cnt, c, r, ctx->cand_dest.p, ctx->cand_prio.p, ctx->s));
            CK(launch_apply(ctx->metric, st, item0, cnt, c, r, ctx->cand_dest.p, ctx->cand_prio.p, ctx->s));
            kernels += 2;
        }
    }
    ctx->sweep_kernels = kernels;
    return ACVD_OK;
}

static int run_sweep(acvd_ctx* ctx, bool timing, bool relaxed, double* eval_ms, int* eval_launches,
                     int64_t* moves) {
    if (timing && (int)ctx->ev_eval.size() != 2 * ctx->nclasses) {
        ctx->drop_graph();
        ctx->drop_events();
        ctx->ev_eval.resize(2 * ctx->nclasses);
        for (auto& e : ctx->ev_eval) CK(cudaEventCreate(&e));
    }
    if (ctx->opts.use_graphs) {
        cudaGraphExec_t& exec = relaxed ? ctx->relaxed_exec : ctx->sweep_exec;
        int64_t& kern = relaxed ? ctx->relaxed_kernels : ctx->exact_kernels;
        if (!exec) {
            cudaGraph_t g;
            const long long before = g_launches;
            CK(cudaStreamBeginCapture(ctx->s, cudaStreamCaptureModeThreadLocal));
            int r = enqueue_sweep(ctx, timing, relaxed);
            cudaError_t e = cudaStreamEndCapture(ctx->s, &g);
            g_launches = before;
            if (r) return r;
            CK(e);
            CK(cudaGraphInstantiate(&exec, g, 0));
            cudaGraphDestroy(g);
            kern = ctx->sweep_kernels;
        }
        CK(cudaGraphLaunch(exec, ctx->s));
        g_launches += kern;
    } else {
        int r = enqueue_sweep(ctx, timing, relaxed);
        if (r) return r;
    }
    int r = sync_counters(ctx);
    if (r) return r;
    *moves = (int64_t)ctx->h_counters[kCntMoves];
    if (timing && !ctx->timing_broken) {
        for (int c = 0; c < ctx->nclasses; c++) {
            if (ctx->sweep_off[c + 1] == ctx->sweep_off[c]) continue;
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ctx->ev_eval[2 * c], ctx->ev_eval[2 * c + 1]) != cudaSuccess) {
                // timing is instrumentation only: report it as unavailable, keep running
                cudaGetLastError();
                ctx->timing_broken = true;
                *eval_ms = -1.0;
                break;
            }
            *eval_ms += ms;
            (*eval_launches)++;
        }
    }
    return ACVD_OK;
}

// The sweeps between two convergence events as one graph: a kernel sets the loop
// and mode conditions, then a WHILE node repeats an IF / ELSE whose bodies are the
// relaxed sweep (+ the energy sum) and the exact sweep, each ending with the
// decision kernel.  Built once per context (dropped with the sweep graphs).
static int build_loop_graph(acvd_ctx* ctx) {
    CK(ctx->dls.resize(1));
    CK(ctx->loop_energy.resize(1));
    // sizes the loop's summation scratch outside the capture
    CK(sum_f64(ctx->energy.p, ctx->K, ctx->loop_energy.p, ctx->loop_scratch, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    int r = ACVD_OK;
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h_loop, h_mode;
    CK(cudaGraphConditionalHandleCreate(&h_loop, g, 0, 0));
    CK(cudaGraphConditionalHandleCreate(&h_mode, g, 0, 0));
    const long long before = g_launches;
    auto fail_capture = [&](int code) {
        cudaGraph_t junk;
        cudaStreamEndCapture(ctx->s, &junk);
        cudaGraphDestroy(g);
        g_launches = before;
        return code;
    };
    CK(cudaStreamBeginCaptureToGraph(ctx->s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    if (launch_loop_start(ctx->dls.p, ctx->dflags.p, h_loop, h_mode, ctx->s) != cudaSuccess)
        return fail_capture(fail(ctx, ACVD_ERR_CUDA, "loop graph: start kernel"));
    cudaGraph_t g2;
    CK(cudaStreamEndCapture(ctx->s, &g2));
    size_t n = 0;
    CK(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> roots(n);
    CK(cudaGraphGetNodes(g, roots.data(), &n));
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    CK(cudaGraphAddNode(&wnode, g, roots.data(), nullptr, n, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = h_mode;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 2;
    cudaGraphNode_t inode;
    CK(cudaGraphAddNode(&inode, body, nullptr, nullptr, 0, &ip));
    for (int b = 0; b < 2; b++) {
        const bool relaxed = b == 0;   // IF body: relaxed sweep; ELSE body: exact sweep
        cudaGraph_t bg = ip.conditional.phGraph_out[b];
        const long long k0 = g_launches;
        CK(cudaStreamBeginCaptureToGraph(ctx->s, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        if ((r = enqueue_sweep(ctx, false, relaxed))) return fail_capture(r);
        if (relaxed && sum_f64(ctx->energy.p, ctx->K, ctx->loop_energy.p, ctx->loop_scratch, ctx->s) != cudaSuccess)
            return fail_capture(fail(ctx, ACVD_ERR_CUDA, "loop graph: energy sum"));
        if (launch_loop_decide(ctx->dls.p, ctx->counters.p, ctx->loop_energy.p, ctx->dflags.p, relaxed, h_loop,
                               h_mode, ctx->s) != cudaSuccess)
            return fail_capture(fail(ctx, ACVD_ERR_CUDA, "loop graph: decision kernel"));
        cudaGraph_t bg2;
        CK(cudaStreamEndCapture(ctx->s, &bg2));
        (relaxed ? ctx->loop_relaxed_kernels : ctx->loop_exact_kernels) = g_launches - k0;
    }
    g_launches = before;
    cudaError_t e = cudaGraphInstantiate(&ctx->loop_exec, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    return ACVD_OK;
}

// Runs the device-side loop from the host's loop state; hl comes back updated.
static int run_sweeps_graph(acvd_ctx* ctx, LoopState& hl, acvd_stats& local) {
    if (!ctx->loop_exec) {
        int r = build_loop_graph(ctx);
        if (r) return r;
    }
    hl.status = 0;
    hl.run = 0;
    hl.relaxed_run = 0;
    hl.moves = 0;
    hl.last_moves = 0;
    hl.eval_ns = 0;
    CK(cudaMemcpyAsync(ctx->dls.p, &hl, sizeof hl, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaGraphLaunch(ctx->loop_exec, ctx->s));
    CK(cudaMemcpyAsync(&hl, ctx->dls.p, sizeof hl, cudaMemcpyDeviceToHost, ctx->s));
    int r = sync_counters(ctx);
    if (r) return r;
    g_launches += 1 + (int64_t)hl.relaxed_run * ctx->loop_relaxed_kernels +
                  (int64_t)(hl.run - hl.relaxed_run) * ctx->loop_exact_kernels;
    local.relaxed_sweeps += hl.relaxed_run;
    local.moves += hl.moves;
    return ACVD_OK;
}

constexpr int kSweepLogCap = 1 << 16;

// Grid of the persistent sweep kernel on this device: every SM times the
// co-resident blocks of the metric's kernel; 0 when cooperative launch is
// unavailable (the per-phase schedule runs instead).
static int sweep_run_grid(acvd_ctx* ctx) {
    if (ctx->run_grid_metric == ctx->metric) return ctx->run_grid;
    int coop = 0, sms = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->opts.device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->opts.device) != cudaSuccess) {
        cudaGetLastError();
        coop = 0;
    }
    const int per_sm = coop ? sweep_run_blocks_per_sm(ctx->metric) : 0;
    ctx->run_grid = coop ? sms * per_sm : 0;
    ctx->run_grid_metric = ctx->metric;
    return ctx->run_grid;
}

// Runs colour sweeps on the device until the host loop's convergence test is
// met (one cooperative launch).  hl carries the loop state in and out.
static int run_sweeps_persistent(acvd_ctx* ctx, LoopState& hl, acvd_stats& local) {
    const int grid = sweep_run_grid(ctx);
    const int64_t per = 2048;
    const int64_t nb = std::max<int64_t>(1, (ctx->K + per - 1) / per);
    CK(ctx->dls.resize(1));
    CK(ctx->dbar.resize(1));
    CK(ctx->esum.resize(nb + (nb + per - 1) / per + 2));
    CK(ctx->doff.resize(ctx->nclasses + 1));
    CK(ctx->slog.resize(kSweepLogCap));
    std::vector<long long> off(ctx->sweep_off.begin(), ctx->sweep_off.end());
    hl.status = 0;
    hl.run = 0;
    hl.relaxed_run = 0;
    hl.moves = 0;
    hl.last_moves = 0;
    hl.eval_ns = 0;
    CK(cudaMemcpyAsync(ctx->dls.p, &hl, sizeof hl, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemsetAsync(ctx->dbar.p, 0, sizeof(GridBar), ctx->s));
    CK(cudaMemcpyAsync(ctx->doff.p, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, ctx->s));
    SweepRun a;
    a.st = ctx->state();
    a.off = ctx->doff.p;
    a.nclasses = ctx->nclasses;
    a.match_rounds = ctx->match_rounds;
    a.cand_dest = ctx->cand_dest.p;
    a.cand_prio = ctx->cand_prio.p;
    a.ls = ctx->dls.p;
    a.bar = ctx->dbar.p;
    a.esum = ctx->esum.p;
    a.log = ctx->slog.p;
    a.log_cap = kSweepLogCap;
    CK(cudaEventRecord(ctx->ev0, ctx->s));
    CK(launch_sweep_run(ctx->metric, a, grid, ctx->s));
    CK(cudaEventRecord(ctx->ev1, ctx->s));
    GridBar hb;
    CK(cudaMemcpyAsync(&hl, ctx->dls.p, sizeof hl, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(&hb, ctx->dbar.p, sizeof hb, cudaMemcpyDeviceToHost, ctx->s));
    int r = sync_counters(ctx);
    if (r) return r;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    local.sweep_kernel_ms += ms;
    local.sweep_kernel_launches += 1;
    local.eval_ms += (double)hl.eval_ns * 1e-6;
    int nonempty = 0;
    for (int c = 0; c < ctx->nclasses; c++) nonempty += ctx->sweep_off[c + 1] > ctx->sweep_off[c];
    local.eval_launches += hl.run * nonempty;
    if (hb.err) return fail(ctx, ACVD_ERR_DEVICE_CHECK, "persistent sweep kernel: a grid barrier wait gave up");
    if (hl.status != 1) return fail(ctx, ACVD_ERR_DEVICE_CHECK, "persistent sweep kernel ended before its loop test");
    return ACVD_OK;
}

// sum of the tracked per-cluster energies (fixed-order FP64 tree)
static int energy_total(acvd_ctx* ctx, double* out) {
    CK(ctx->dtmp.resize(2));
    CK(sum_f64(ctx->energy.p, ctx->K, ctx->dtmp.p, ctx->scratch, ctx->s));
    CK(cudaMemcpyAsync(out, ctx->dtmp.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

// Algorithmic bytes of the evaluation kernels from the device counters: per visited
// item its boundary flag; per screened item its 8-slot ring, label and evaluation
// sweep; per ring slot the neighbour's label; per cached screen its 16-byte record
// (cluster, targets, evaluation sweep) and up to 4 cluster stamps; per boundary item its record, its
// cluster's record and size; per destination cluster its record; per proposal the
// candidate slots and two claim words.
static int64_t eval_bytes_of(const acvd_ctx* ctx, const unsigned long long* c) {
    const int64_t R = ctx->metric == kIso ? 16 : (ctx->metric == kQEM ? 40 : 64);
    const int64_t C = 16 * (int64_t)ev_stride(ctx->metric);
    return 1 * (int64_t)c[kCntVisited] + 40 * (int64_t)c[kCntScreened] + 32 * (int64_t)c[kCntCached] +
           4 * (int64_t)c[kCntSlots] + (R + C + 4) * (int64_t)c[kCntBoundary] + C * (int64_t)c[kCntTargets] +
           24 * (int64_t)c[kCntCand];
}

// the per-sweep log's snapshot of the cumulative counters
struct SweepCounters {
    unsigned long long c[kNumCounters] = {};
    void take(const acvd_ctx* ctx) {
        for (int q = 0; q < kNumCounters; q++) c[q] = ctx->h_counters[q];
    }
    long long d(const SweepCounters& o, int q) const { return (long long)(c[q] - o.c[q]); }
    int64_t eval_bytes(const acvd_ctx* ctx) const { return eval_bytes_of(ctx, c); }
};

struct SweepLogFile {
    FILE* f = nullptr;
    explicit SweepLogFile(const char* path) {
        if (path && *path) f = std::fopen(path, "a");
    }
    ~SweepLogFile() {
        if (f) std::fclose(f);
    }
};

extern "C" int acvd_minimize(acvd_ctx* ctx, acvd_stats* stats) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh || !ctx->ready_metric || !ctx->ready_labels)
        return fail(ctx, ACVD_ERR_ARG, "acvd_minimize needs acvd_set_mesh, acvd_set_metric and acvd_set_labels");
    CK(cudaSetDevice(ctx->opts.device));
    acvd_stats local;
    std::memset(&local, 0, sizeof local);
    // ACVD_SWEEP_LOG=<path>: one JSON line per sweep and per convergence event is
    // appended to the file (the sweeps run from the host, with CUDA events around
    // every evaluation kernel); an observation mode, the clustering is unchanged
    const char* log_path = std::getenv("ACVD_SWEEP_LOG");
    SweepLogFile slog(log_path);
    const bool timing = ctx->opts.kernel_timing != 0 || slog.f != nullptr;
    // ProcessClustering: the unconstrained first phase of the QEM metric (:683-688)
    ctx->flags.constrained = (ctx->metric == kQEM && ctx->unconstrained) ? 0 : 1;
    ctx->flags.connexity = 0;
    ctx->flags.level = ctx->level;
    ctx->flags.thr = 1e-3f;
    int r = upload_flags(ctx);
    if (r) return r;
    CK(cudaMemsetAsync(ctx->counters.p, 0, kCounterWords * sizeof(unsigned long long), ctx->s));
    const long long launches0 = g_launches;
    cudaEvent_t t0, t1;
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    CK(cudaEventRecord(t0, ctx->s));
    int status = ACVD_OK;
    do {
        // FillHolesInClustering, FillQueuesFromClustering, ReComputeStatistics (:727-730)
        if (cudaMemsetAsync(ctx->evald.p, 0xff, ctx->nV * sizeof(int), ctx->s) != cudaSuccess ||
            cudaMemsetAsync(ctx->stamp.p, 0, (ctx->K + 1) * sizeof(int), ctx->s) != cudaSuccess) {
            status = fail(ctx, ACVD_ERR_CUDA, "memset of the activity arrays failed");
            break;
        }
        if ((r = set_sweep_state(ctx, 0, 0))) { status = r; break; }
        if (cudaMemsetAsync(ctx->fx_delta.p, 0, (size_t)(ctx->K + 1) * acc_stride(kAniso) * sizeof(long long), ctx->s) ||
            cudaMemsetAsync(ctx->out_cnt.p, 0, (ctx->K + 1) * sizeof(int), ctx->s) ||
            cudaMemsetAsync(ctx->in_done.p, 0, (ctx->K + 1) * sizeof(int), ctx->s) ||
            cudaMemsetAsync(ctx->out_done.p, 0, (ctx->K + 1) * sizeof(int), ctx->s)) {
            status = fail(ctx, ACVD_ERR_CUDA, "memset of the relaxed-step arrays failed");
            break;
        }
        int unassigned = 0;
        if ((r = fill_holes(ctx, &unassigned))) { status = r; break; }
        if ((r = recompute(ctx))) { status = r; break; }
        // items of non-frozen clusters, the base of the early-convergence test (:733-736)
        int64_t early = ctx->nV - unassigned;
        if (ctx->has_frozen) {
            std::vector<int> h_size(ctx->K);
            if (cudaMemcpyAsync(h_size.data(), ctx->size.p, ctx->K * sizeof(int), cudaMemcpyDeviceToHost, ctx->s) !=
                    cudaSuccess ||
                cudaStreamSynchronize(ctx->s) != cudaSuccess) {
                status = fail(ctx, ACVD_ERR_CUDA, "reading the cluster sizes failed");
                break;
            }
            early = 0;
            for (int c = 0; c < ctx->K; c++)
                if (!ctx->h_frozen[c]) early += h_size[c];
        }
        int convergences = 0;
        int sweeps = 0;
        // relaxed sweeps while the connectivity constraint is off; back to exact
        // claims for the rest of a phase as soon as a relaxed sweep raises the energy
        bool relaxed_ok = ctx->use_relaxed;
        double e_prev = 0.0;
        bool have_prev = false;
        if (relaxed_ok && (r = energy_total(ctx, &e_prev))) { status = r; break; }
        have_prev = relaxed_ok;
        const bool trace = std::getenv("ACVD_TRACE") != nullptr;
        auto t_trace = std::chrono::steady_clock::now();
        const bool persistent = ctx->opts.persistent && sweep_run_grid(ctx) > 0;
        // graph-looped sweeps unless per-sweep events or the per-sweep trace are wanted
        const bool device_loop = !persistent && !timing && !trace && ctx->opts.use_graphs &&
                                 std::getenv("ACVD_HOST_LOOP") == nullptr;
        if (slog.f && persistent) {
            status = fail(ctx, ACVD_ERR_UNSUPPORTED, "ACVD_SWEEP_LOG needs the per-phase schedule");
            break;
        }
        SweepCounters prev_ctr;
        if (slog.f) {
            if ((r = sync_counters(ctx))) { status = r; break; }
            prev_ctr.take(ctx);
        }
        for (;;) {
            int64_t mods = 0;
            const bool relaxed = relaxed_ok && !ctx->flags.connexity;
            if (persistent) {
                // every sweep up to the next convergence test, on the device
                LoopState hl;
                std::memset(&hl, 0, sizeof hl);
                hl.early = early;
                hl.sweeps = sweeps;
                hl.max_loops = ctx->opts.max_loops;
                hl.convergences = convergences;
                hl.relaxed_ok = relaxed_ok ? 1 : 0;
                hl.have_prev = have_prev ? 1 : 0;
                hl.e_prev = e_prev;
                if ((r = run_sweeps_persistent(ctx, hl, local))) { status = r; break; }
                if (trace) {
                    const int first = sweeps, last = std::min(hl.sweeps, kSweepLogCap);
                    std::vector<SweepLog> lg(std::max(0, last - first));
                    if (!lg.empty() &&
                        cudaMemcpy(lg.data(), ctx->slog.p + first, lg.size() * sizeof(SweepLog),
                                   cudaMemcpyDeviceToHost) != cudaSuccess) {
                        status = fail(ctx, ACVD_ERR_CUDA, "trace log copy failed");
                        break;
                    }
                    const auto now = std::chrono::steady_clock::now();
                    std::fprintf(stderr, "acvd persistent run: sweeps %d-%d in %.3f ms (device eval %.3f ms)\n",
                                 first + 1, hl.sweeps, std::chrono::duration<double, std::milli>(now - t_trace).count(),
                                 hl.eval_ns * 1e-6);
                    for (size_t q = 0; q < lg.size(); q++)
                        std::fprintf(stderr, "acvd sweep %d %s moves %lld energy %.17g conv %d flags %d%d\n",
                                     first + 1 + (int)q, lg[q].relaxed ? "relaxed" : "exact", lg[q].moves,
                                     lg[q].energy, convergences, ctx->flags.constrained, ctx->flags.connexity);
                    t_trace = now;
                }
                sweeps = hl.sweeps;
                relaxed_ok = hl.relaxed_ok != 0;
                have_prev = hl.have_prev != 0;
                e_prev = hl.e_prev;
                local.relaxed_sweeps += hl.relaxed_run;
                local.moves += hl.moves;
                mods = hl.last_moves;
            } else if (device_loop) {
                // every sweep up to the next convergence test, looped on the device by the graph
                LoopState hl;
                std::memset(&hl, 0, sizeof hl);
                hl.early = early;
                hl.sweeps = sweeps;
                hl.max_loops = ctx->opts.max_loops;
                hl.convergences = convergences;
                hl.relaxed_ok = relaxed_ok ? 1 : 0;
                hl.have_prev = have_prev ? 1 : 0;
                hl.e_prev = e_prev;
                if ((r = run_sweeps_graph(ctx, hl, local))) { status = r; break; }
                sweeps = hl.sweeps;
                relaxed_ok = hl.relaxed_ok != 0;
                have_prev = hl.have_prev != 0;
                e_prev = hl.e_prev;
                mods = hl.last_moves;
            } else {
            const double eval_ms0 = local.eval_ms;
            const auto t_sweep = std::chrono::steady_clock::now();
            if ((r = run_sweep(ctx, timing, relaxed, &local.eval_ms, &local.eval_launches, &mods))) { status = r; break; }
            double e_now = 0.0;
            if (relaxed) {
                local.relaxed_sweeps++;
                if ((r = energy_total(ctx, &e_now))) { status = r; break; }
                if (have_prev && !(e_now < e_prev)) relaxed_ok = false;
                e_prev = e_now;
                have_prev = true;
            }
            sweeps++;
            local.moves += mods;
            if (slog.f) {
                const double sweep_ms =
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_sweep).count();
                if (!relaxed && (r = energy_total(ctx, &e_now))) { status = r; break; }
                SweepCounters now_ctr;
                now_ctr.take(ctx);
                const double ems = local.eval_ms - eval_ms0;
                const int64_t bytes = now_ctr.eval_bytes(ctx) - prev_ctr.eval_bytes(ctx);
                std::fprintf(slog.f,
                             "{\"sweep\": %d, \"mode\": \"%s\", \"moves\": %lld, \"candidates\": %lld, "
                             "\"boundary_items\": %lld, \"targets\": %lld, \"visited\": %lld, \"screened\": %lld, "
                             "\"cached\": %lld, \"reverted\": %lld, \"energy\": %.17g, \"eval_ms\": %.6f, "
                             "\"eval_bytes\": %lld, \"eval_gbs\": %.3f, \"sweep_ms\": %.6f, \"constrained\": %d, "
                             "\"connexity\": %d, \"convergences\": %d}\n",
                             sweeps, relaxed ? "relaxed" : "exact", (long long)mods,
                             now_ctr.d(prev_ctr, kCntCand), now_ctr.d(prev_ctr, kCntBoundary),
                             now_ctr.d(prev_ctr, kCntTargets), now_ctr.d(prev_ctr, kCntVisited),
                             now_ctr.d(prev_ctr, kCntScreened), now_ctr.d(prev_ctr, kCntCached),
                             now_ctr.d(prev_ctr, kCntReverted), e_now, ems, (long long)bytes,
                             ems > 0 ? bytes / (ems * 1e6) : 0.0, sweep_ms, ctx->flags.constrained,
                             ctx->flags.connexity, convergences);
                prev_ctr = now_ctr;
            }
            }
            if (trace && !persistent && !device_loop) {
                const auto now = std::chrono::steady_clock::now();
                std::fprintf(stderr,
                             "acvd sweep %d %s %.3f ms moves %lld cand %llu boundary %llu targets %llu visited %llu "
                             "screened %llu cached %llu reverted %llu conv %d flags %d%d\n",
                             sweeps, relaxed ? "relaxed" : "exact",
                             std::chrono::duration<double, std::milli>(now - t_trace).count(), (long long)mods,
                             ctx->h_counters[kCntCand], ctx->h_counters[kCntBoundary], ctx->h_counters[kCntTargets],
                             ctx->h_counters[kCntVisited], ctx->h_counters[kCntScreened], ctx->h_counters[kCntCached],
                             ctx->h_counters[kCntReverted], convergences,
                             ctx->flags.constrained, ctx->flags.connexity);
                t_trace = now;
            }
            if (mods == 0 || sweeps > ctx->opts.max_loops || (mods <= early / 1000 && convergences <= 1)) {
                bool flags_changed = false;
                if (ctx->unconstrained && convergences == 0 && ctx->metric == kQEM) {
                    ctx->flags.constrained = 1;
                    flags_changed = true;
                }
                if (convergences >= 1 && !ctx->flags.connexity) {
                    ctx->flags.connexity = 1;
                    flags_changed = true;
                }
                if (slog.f) {
                    // the incrementally tracked energy (FP32 items, double-float records)
                    // against a full FP64 recompute of the same clustering
                    double e_tracked = 0.0, e_fp64 = 0.0;
                    if ((r = energy_total(ctx, &e_tracked)) || (r = recompute(ctx)) ||
                        (r = energy_total(ctx, &e_fp64))) { status = r; break; }
                    std::fprintf(slog.f,
                                 "{\"event\": \"convergence\", \"sweep\": %d, \"convergence\": %d, "
                                 "\"energy_tracked\": %.17g, \"energy_fp64\": %.17g, \"rel_err\": %.6g}\n",
                                 sweeps, convergences + 1, e_tracked, e_fp64,
                                 e_fp64 != 0.0 ? std::fabs(e_tracked - e_fp64) / std::fabs(e_fp64) : 0.0);
                }
                if (flags_changed && (r = upload_flags(ctx))) { status = r; break; }
                convergences++;
                int disc = 0;
                if ((r = clean(ctx, &disc))) { status = r; break; }
                int un = 0;
                if ((r = fill_holes(ctx, &un))) { status = r; break; }
                local.disconnected = disc;
                local.unassigned = un;
                if ((r = recompute(ctx))) { status = r; break; }
                // SetAllClustersToModified (:822): every item is evaluated again
                if ((r = set_sweep_state(ctx, sweeps, sweeps))) { status = r; break; }
                relaxed_ok = ctx->use_relaxed;
                have_prev = false;
                if (relaxed_ok && !ctx->flags.connexity) {
                    if ((r = energy_total(ctx, &e_prev))) { status = r; break; }
                    have_prev = true;
                }
                if (disc == 0 && mods == 0) break;
                // MaxNumberOfLoops ends the minimisation like a convergence (:803-810)
                if (sweeps >= ctx->opts.max_loops) { local.hit_loop_cap = 1; break; }
                if (convergences >= ctx->opts.max_convergences) break;
            }
        }
        local.sweeps = sweeps;
        local.convergences = convergences;
    } while (0);
    CK(cudaEventRecord(t1, ctx->s));
    CK(cudaEventSynchronize(t1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, t0, t1));
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    local.device_ms = ms;
    r = sync_counters(ctx);
    if (r) return r;
    local.candidates = (int64_t)ctx->h_counters[kCntCand];
    local.boundary_items = (int64_t)ctx->h_counters[kCntBoundary];
    local.targets = (int64_t)ctx->h_counters[kCntTargets];
    local.visited = (int64_t)ctx->h_counters[kCntVisited];
    local.slots = (int64_t)ctx->h_counters[kCntSlots];
    local.kernel_launches = g_launches - launches0;
    if (ctx->h_counters[kCntError] && status == ACVD_OK)
        status = fail(ctx, ACVD_ERR_DEVICE_CHECK,
                      std::to_string(ctx->h_counters[kCntError]) + " device-side index checks failed");
    local.reverted = (int64_t)ctx->h_counters[kCntReverted];
    local.eval_bytes = eval_bytes_of(ctx, ctx->h_counters);
    if (status == ACVD_OK) {
        // every way out of the loop follows a convergence event, whose recompute left
        // the per-cluster FP64 energies of the final labels in place
        double et = 0.0;
        int rr = energy_total(ctx, &et);
        if (rr) return rr;
        local.energy = et;
    }
    if (stats) *stats = local;
    return status;
}

extern "C" int acvd_get_labels(acvd_ctx* ctx, int32_t* labels) {
    if (!ctx || !labels) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "no labels");
    CK(cudaSetDevice(ctx->opts.device));
    CK(ctx->label_orig.resize(ctx->nV));
    CK(launch_gather_i32(ctx->label.p, ctx->inv.p, ctx->nV, ctx->label_orig.p, ctx->s));
    CK(cudaMemcpyAsync(labels, ctx->label_orig.p, ctx->nV * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

// Accumulators and evaluation records for the current labels (recomputed).
extern "C" int acvd_get_clusters(acvd_ctx* ctx, int32_t* sizes, double* S, double* W, double* quadric,
                                 double* centroid, double* energy, double* energy_total) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_metric || !ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "no metric or labels");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->flags.level = ctx->level;
    int r = upload_flags(ctx);
    if (r) return r;
    r = recompute(ctx);
    if (r) return r;
    const int K = ctx->K;
    const int as = acc_stride(ctx->metric);
    // the accumulators come back only when one of their views is asked for
    const bool want_acc = S || W || quadric;
    std::vector<df> acc(want_acc ? (size_t)K * as : 0);
    if (want_acc)
        CK(cudaMemcpyAsync(acc.data(), ctx->acc.p, acc.size() * sizeof(df), cudaMemcpyDeviceToHost, ctx->s));
    if (sizes) CK(cudaMemcpyAsync(sizes, ctx->size.p, K * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    if (energy) CK(cudaMemcpyAsync(energy, ctx->energy.p, K * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    if (energy_total) {
        CK(ctx->dtmp.resize(2));
        CK(sum_f64(ctx->energy.p, K, ctx->dtmp.p, ctx->scratch, ctx->s));
        CK(cudaMemcpyAsync(energy_total, ctx->dtmp.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    }
    if (centroid) {
        DBuf<double> c;
        CK(c.resize(3 * (size_t)K));
        CK(launch_centroids(ctx->metric, ctx->state(), c.p, ctx->s));
        CK(cudaMemcpyAsync(centroid, c.p, 3 * (size_t)K * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    CK(cudaStreamSynchronize(ctx->s));
    for (int k = 0; want_acc && k < K; k++) {
        const df* a = acc.data() + (size_t)k * as;
        auto d = [](df x) { return (double)x.hi + (double)x.lo; };
        if (S) for (int j = 0; j < 3; j++) S[3 * k + j] = d(a[j]);
        if (W) W[k] = d(a[3]);
        if (quadric) {
            double* q = quadric + 9 * (size_t)k;
            if (ctx->metric == kIso) {
                for (int j = 0; j < 9; j++) q[j] = 0.0;
            } else {
                // the reference's compact quadric: A entries and -b in slots 3, 6, 8
                q[0] = d(a[4]); q[1] = d(a[5]); q[2] = d(a[6]); q[3] = -d(a[10]);
                q[4] = d(a[7]); q[5] = d(a[8]); q[6] = -d(a[11]); q[7] = d(a[9]); q[8] = -d(a[12]);
            }
        }
    }
    return ACVD_OK;
}

extern "C" int acvd_get_mesh_energies(acvd_ctx* ctx, double* energies) {
    if (!ctx || !energies) return ACVD_ERR_ARG;
    if (ctx->nmesh == 0) return fail(ctx, ACVD_ERR_ARG, "no batch set");
    double tot = 0.0;
    int r = acvd_get_clusters(ctx, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &tot);
    if (r) return r;
    // per-mesh totals in the same fixed order as the global one
    for (int m = 0; m < ctx->nmesh; m++) {
        const int64_t a = ctx->h_koff[m], b = ctx->h_koff[m + 1];
        CK(ctx->dtmp.resize(2));
        CK(sum_f64(ctx->energy.p + a, b - a, ctx->dtmp.p, ctx->scratch, ctx->s));
        CK(cudaMemcpyAsync(&energies[m], ctx->dtmp.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    return ACVD_OK;
}

extern "C" int acvd_get_boundary_edges(acvd_ctx* ctx, int32_t* ids, int64_t* count) {
    if (!ctx || !count) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "no labels");
    CK(cudaSetDevice(ctx->opts.device));
    const int64_t ne = ctx->nE;
    DBuf<uint32_t> flags, pos;
    DBuf<int> out;
    CK(flags.resize(ne + 1));
    CK(pos.resize(ne + 1));
    CK(ctx->dtmp.resize(2));
    uint32_t* total = (uint32_t*)ctx->dtmp.p;
    CK(launch_boundary_edges(ctx->edge_int.p, ne, ctx->label.p, flags.p, ctx->s));
    CK(exclusive_scan_u32(flags.p, pos.p, ne, total, ctx->scratch, ctx->s));
    uint32_t t = 0;
    CK(cudaMemcpyAsync(&t, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    *count = t;
    if (ids && t) {
        CK(out.resize(t));
        CK(launch_compact(flags.p, pos.p, ne, out.p, ctx->s));
        CK(cudaMemcpyAsync(ids, out.p, t * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    return ACVD_OK;
}

// Curvature of vertex clustering (vtkDiscreteRemeshing.h:630-637 ->
// vtkCurvatureMeasure, polynomial fitting on the vertex 3-ring): indicator[nV]
// and principal_dirs[6 nV], either may be NULL.
extern "C" int acvd_compute_curvature(acvd_ctx* ctx, double* indicator, float* principal_dirs) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_mesh) return fail(ctx, ACVD_ERR_ARG, "acvd_compute_curvature before acvd_set_mesh");
    CK(cudaSetDevice(ctx->opts.device));
    const int64_t nv = ctx->nV, ne = ctx->nE;
    CK(ctx->curv_poly.resize(ne));
    CK(ctx->curv_slot.resize(2 * ne));
    CK(ctx->curv_ind.resize(nv));
    CK(ctx->curv_dirs.resize(6 * nv));
    CK(ctx->dtmp.resize(2));
    unsigned long long* overflow = (unsigned long long*)ctx->dtmp.p;
    CK(cudaMemsetAsync(overflow, 0, sizeof(unsigned long long), ctx->s));
    CK(ctx->curv_faces.resize(curvature_face_bytes(ctx->nF)));
    CK(launch_curvature(ctx->xyz.p, ctx->tri.p, nv, ctx->nF, ne, ctx->edge_v.p, ctx->edge_int.p, ctx->vf_row.p,
                        ctx->vf_face.p, ctx->row.p, ctx->col.p, ctx->perm.p, ctx->inv.p, ctx->curv_poly.p,
                        ctx->curv_slot.p, ctx->curv_faces.p, ctx->curv_ind.p, ctx->curv_dirs.p, overflow, ctx->s));
    unsigned long long h_over = 0;
    CK(cudaMemcpyAsync(&h_over, overflow, sizeof h_over, cudaMemcpyDeviceToHost, ctx->s));
    if (indicator)
        CK(cudaMemcpyAsync(indicator, ctx->curv_ind.p, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    if (principal_dirs)
        CK(cudaMemcpyAsync(principal_dirs, ctx->curv_dirs.p, 6 * nv * sizeof(float), cudaMemcpyDeviceToHost,
                           ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (h_over)
        return fail(ctx, ACVD_ERR_UNSUPPORTED,
                    std::to_string(h_over) + " vertices have a 3-ring larger than the curvature kernel's buffers");
    return ACVD_OK;
}

// One level of midpoint subdivision (vtkSurface::Subdivide, Common/vtkSurface.cxx:605-677)
// with the parent interpolation of the indicator (vtkDiscreteRemeshing.h:731-745).
// Independent of the context's mesh: the context gives the device and the stream.
extern "C" int acvd_subdivide(acvd_ctx* ctx, int64_t n_vertices, const double* xyz, int64_t n_faces,
                              const int32_t* tri, const int32_t* csr_row, const int32_t* csr_col, int64_t n_edges,
                              const int32_t* edge_v, const double* indicator, double* out_xyz, int32_t* out_tri,
                              int32_t* parent1, int32_t* parent2, double* out_indicator) {
    if (!ctx) return ACVD_ERR_ARG;
    if (n_vertices < 0 || n_faces < 0 || n_edges < 0 || !xyz || !tri || !csr_row || !csr_col || !edge_v ||
        !out_xyz || !out_tri || !parent1 || !parent2)
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide: null or negative argument");
    if ((indicator == nullptr) != (out_indicator == nullptr))
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide: indicator and out_indicator go together");
    if (n_vertices + n_edges > INT32_MAX || 4 * n_faces > INT32_MAX)
        return fail(ctx, ACVD_ERR_UNSUPPORTED, "acvd_subdivide: the subdivided mesh exceeds 32-bit ids");
    if (csr_row[n_vertices] != 2 * n_edges)
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide: ring CSR does not hold 2 n_edges slots");
    // vtkSurface::Subdivide skips inactive faces (first two corners equal); this
    // build keeps the 4 f .. 4 f + 3 numbering and rejects them instead
    for (int64_t f = 0; f < n_faces; f++)
        if (tri[3 * f] == tri[3 * f + 1])
            return fail(ctx, ACVD_ERR_UNSUPPORTED, "acvd_subdivide: face " + std::to_string(f) + " is degenerate");
    CK(cudaSetDevice(ctx->opts.device));
    const int64_t nv = n_vertices, nf = n_faces, ne = n_edges, nout = n_vertices + n_edges;
    DBuf<double> d_xyz, d_ind, d_oxyz, d_oind;
    DBuf<int> d_tri, d_row, d_col, d_ev, d_otri, d_p1, d_p2;
    DBuf<int4> d_work;
    CK(d_xyz.resize(3 * nv)); CK(d_tri.resize(3 * nf)); CK(d_row.resize(nv + 1)); CK(d_col.resize(2 * ne));
    CK(d_ev.resize(2 * ne)); CK(d_oxyz.resize(3 * nout)); CK(d_otri.resize(12 * nf));
    CK(d_p1.resize(ne)); CK(d_p2.resize(ne));
    CK(d_work.resize((acvd_subdivide_work_bytes(ne) + 15) / 16));
    if (indicator) { CK(d_ind.resize(nv)); CK(d_oind.resize(nout)); }
    CK(cudaMemcpyAsync(d_xyz.p, xyz, 3 * nv * sizeof(double), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_tri.p, tri, 3 * nf * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_row.p, csr_row, (nv + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_col.p, csr_col, 2 * ne * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(d_ev.p, edge_v, 2 * ne * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    if (indicator) CK(cudaMemcpyAsync(d_ind.p, indicator, nv * sizeof(double), cudaMemcpyHostToDevice, ctx->s));
    int r = acvd_subdivide_device(ctx, nv, d_xyz.p, nf, d_tri.p, d_row.p, d_col.p, ne, d_ev.p, d_ind.p, d_oxyz.p,
                                  d_otri.p, d_p1.p, d_p2.p, d_oind.p, d_work.p);
    if (r) return r;
    unsigned int missing = 0;
    CK(cudaMemcpyAsync(&missing, (const int*)d_work.p + 2 * ne, sizeof missing, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(out_xyz, d_oxyz.p, 3 * nout * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(out_tri, d_otri.p, 12 * nf * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(parent1, d_p1.p, ne * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(parent2, d_p2.p, ne * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    if (indicator)
        CK(cudaMemcpyAsync(out_indicator, d_oind.p, nout * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (missing)
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide: " + std::to_string(missing) +
                                            " faces refer to a missing vertex or to an edge missing from the ring CSR");
    return ACVD_OK;
}

// Work bytes of acvd_subdivide_device: the ring slots' edge ids and the fault count.
extern "C" int64_t acvd_subdivide_work_bytes(int64_t n_edges) {
    return 2 * n_edges * (int64_t)sizeof(int) + 16;
}

// acvd_subdivide on device buffers, enqueued on the context's stream (no
// allocation, no synchronisation).  The count of faces with an edge missing from
// the ring CSR lands in the uint32 at d_work + 2 n_edges ints.
extern "C" int acvd_subdivide_device(acvd_ctx* ctx, int64_t n_vertices, const double* d_xyz, int64_t n_faces,
                                     const int32_t* d_tri, const int32_t* d_row, const int32_t* d_col,
                                     int64_t n_edges, const int32_t* d_edge_v, const double* d_ind,
                                     double* d_out_xyz, int32_t* d_out_tri, int32_t* d_parent1,
                                     int32_t* d_parent2, double* d_out_ind, void* d_work) {
    if (!ctx) return ACVD_ERR_ARG;
    if (n_vertices < 0 || n_faces < 0 || n_edges < 0 || !d_xyz || !d_tri || !d_row || !d_col || !d_edge_v ||
        !d_out_xyz || !d_out_tri || !d_parent1 || !d_parent2 || !d_work)
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide_device: null or negative argument");
    if ((d_ind == nullptr) != (d_out_ind == nullptr))
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide_device: d_ind and d_out_ind go together");
    if (n_vertices + n_edges > INT32_MAX || 4 * n_faces > INT32_MAX)
        return fail(ctx, ACVD_ERR_UNSUPPORTED, "acvd_subdivide_device: the subdivided mesh exceeds 32-bit ids");
    if ((reinterpret_cast<uintptr_t>(d_work) & 15u) != 0)
        return fail(ctx, ACVD_ERR_ARG, "acvd_subdivide_device: d_work must be 16-byte aligned");
    CK(cudaSetDevice(ctx->opts.device));
    int* slot = (int*)d_work;
    unsigned int* missing = (unsigned int*)(slot + 2 * n_edges);
    CK(cudaMemsetAsync(missing, 0, sizeof(unsigned int), ctx->s));
    CK(launch_subdivide(d_xyz, n_vertices, d_tri, n_faces, d_row, d_col, d_edge_v, n_edges, d_ind, slot, d_out_xyz,
                        d_out_tri, d_parent1, d_parent2, d_out_ind, missing, ctx->s));
    return ACVD_OK;
}

// ACVD's quadric post-placement of the output vertices (ACVD.cxx:217-291) for the
// current clustering; points: 3K doubles.
extern "C" int acvd_post_placement(acvd_ctx* ctx, int level, double* points) {
    if (!ctx || !points) return ACVD_ERR_ARG;
    if (!ctx->ready_metric || !ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "no metric or labels");
    if (level < 0 || level > 3) return fail(ctx, ACVD_ERR_ARG, "acvd_post_placement: level outside [0, 3]");
    CK(cudaSetDevice(ctx->opts.device));
    ctx->flags.level = ctx->level;
    int r = upload_flags(ctx);
    if (r) return r;
    r = recompute(ctx);
    if (r) return r;
    const int64_t nv = ctx->nV;
    const int K = ctx->K;
    // the output vertices before placement: the metric's cluster centroids
    DBuf<double> start, qv, out;
    CK(start.resize(3 * (size_t)K));
    CK(launch_centroids(ctx->metric, ctx->state(), start.p, ctx->s));
    // items by cluster, in original vertex ids
    CK(ctx->label_orig.resize(nv));
    CK(launch_gather_i32(ctx->label.p, ctx->inv.p, nv, ctx->label_orig.p, ctx->s));
    DevState st = ctx->state();
    st.label = ctx->label_orig.p;
    CK(ctx->wk_a.resize(nv)); CK(ctx->wk_b.resize(nv)); CK(ctx->wk_c.resize(nv)); CK(ctx->wk_d.resize(nv));
    CK(ctx->wk_cnt.resize(K + 1)); CK(ctx->wk_off.resize(K + 1));
    CK(cudaMemsetAsync(ctx->wk_cnt.p, 0, (K + 1) * sizeof(uint32_t), ctx->s));
    CK(launch_cluster_keys(st, ctx->wk_a.p, ctx->wk_b.p, ctx->wk_cnt.p, ctx->s));
    CK(radix_sort_pairs(ctx->wk_a.p, ctx->wk_b.p, ctx->wk_c.p, ctx->wk_d.p, nv, bits_for((uint64_t)K), ctx->scratch,
                        ctx->s));
    CK(exclusive_scan_u32(ctx->wk_cnt.p, ctx->wk_off.p, K + 1, nullptr, ctx->scratch, ctx->s));
    CK(qv.resize(9 * (size_t)nv));
    CK(launch_vertex_quadrics(ctx->xyz.p, ctx->tri.p, ctx->vf_row.p, ctx->vf_face.p, nv, qv.p, ctx->s));
    CK(out.resize(3 * (size_t)K));
    CK(ctx->dtmp.resize(2));
    CK(launch_post_place(qv.p, ctx->wk_b.p, ctx->wk_off.p, ctx->wk_cnt.p, (const int*)ctx->wk_cnt.p, (int*)ctx->dtmp.p,
                         start.p, K, level, out.p, ctx->s));
    CK(cudaMemcpyAsync(points, out.p, 3 * (size_t)K * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

// The dual mesh's triangles on the device (cluster ids), *n_tris of them in `out`.
static int build_dual(acvd_ctx* ctx, DBuf<int>& out, int64_t* n_tris) {
    const int64_t nf = ctx->nF;
    DBuf<uint32_t> flags, pos, klo, khi, order, t1, t2, keep, kpos;
    DBuf<int> faces, sel;
    CK(flags.resize(nf + 1));
    CK(pos.resize(nf + 1));
    CK(ctx->dtmp.resize(2));
    uint32_t* total = (uint32_t*)ctx->dtmp.p;
    CK(launch_dual_faces(ctx->tri_int.p, nf, ctx->label.p, ctx->K, flags.p, ctx->s));
    CK(exclusive_scan_u32(flags.p, pos.p, nf, total, ctx->scratch, ctx->s));
    uint32_t m = 0;
    CK(cudaMemcpyAsync(&m, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    if (m == 0) { *n_tris = 0; return ACVD_OK; }
    CK(faces.resize(m));
    CK(launch_compact(flags.p, pos.p, nf, faces.p, ctx->s));
    CK(klo.resize(m)); CK(khi.resize(m)); CK(order.resize(m)); CK(t1.resize(m)); CK(t2.resize(m));
    CK(keep.resize(m + 1)); CK(kpos.resize(m + 1));
    CK(launch_dual_keys(ctx->tri_int.p, faces.p, m, ctx->label.p, klo.p, khi.p, order.p, ctx->s));
    // stable LSD sort on (khi, klo): by klo first, then by khi
    CK(radix_sort_pairs(klo.p, order.p, t1.p, t2.p, m, 32, ctx->scratch, ctx->s));
    CK(launch_gather_u32(khi.p, order.p, m, t1.p, ctx->s));           // khi in klo-sorted order
    CK(cudaMemcpyAsync(khi.p, t1.p, m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->s));
    // carry klo along the second pass through a permutation index
    DBuf<uint32_t> perm, klo2;
    CK(perm.resize(m)); CK(klo2.resize(m));
    {
        std::vector<uint32_t> io(m);
        for (uint32_t j = 0; j < m; j++) io[j] = j;
        CK(cudaMemcpyAsync(perm.p, io.data(), m * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    CK(radix_sort_pairs(khi.p, perm.p, t1.p, t2.p, m, 31, ctx->scratch, ctx->s));
    CK(launch_gather_u32(klo.p, perm.p, m, klo2.p, ctx->s));
    CK(launch_gather_u32(order.p, perm.p, m, t1.p, ctx->s));
    CK(launch_dual_unique(klo2.p, khi.p, t1.p, m, keep.p, ctx->s));
    CK(exclusive_scan_u32(keep.p, kpos.p, m, total, ctx->scratch, ctx->s));
    uint32_t t = 0;
    CK(cudaMemcpyAsync(&t, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    *n_tris = t;
    if (t) {
        CK(sel.resize(t));
        CK(out.resize(3 * (size_t)t));
        CK(launch_compact(keep.p, kpos.p, m, sel.p, ctx->s));
        CK(launch_dual_write(ctx->tri_int.p, faces.p, sel.p, t, ctx->label.p, out.p, ctx->s));
    }
    return ACVD_OK;
}

// One pass of vtkDiscreteRemeshing::DetectNonManifoldOutputVertices
// (DiscreteRemeshing/vtkDiscreteRemeshing.h:165-383) on the current clustering.
// The device finds the clusters whose output vertex is not manifold and which hold
// no non-manifold input vertex, and their output-mesh neighbours; the host then
// adds the new clusters in the reference's order (an item is taken from the cluster,
// or from a neighbour's cluster when it has a single item) and freezes every other
// cluster.  The next acvd_minimize is the reference's re-entry into MinimizeEnergy.
extern "C" int acvd_force_manifold_step(acvd_ctx* ctx, int32_t* n_issues, int32_t* n_clusters) {
    if (!ctx || !n_issues || !n_clusters) return ACVD_ERR_ARG;
    if (!ctx->ready_metric || !ctx->ready_labels)
        return fail(ctx, ACVD_ERR_ARG, "acvd_force_manifold_step needs a metric and a clustering");
    CK(cudaSetDevice(ctx->opts.device));
    *n_issues = 0;
    *n_clusters = ctx->K;
    int r = recompute(ctx);   // current cluster sizes
    if (r) return r;
    DBuf<int> dt;
    int64_t t = 0;
    if ((r = build_dual(ctx, dt, &t))) return r;
    const int K = ctx->K;
    const int64_t nv = ctx->nV, ne = ctx->nE;
    DBuf<unsigned> cnt, off, cursor;
    DBuf<int> list;
    DBuf<unsigned char> bad, has_nm, issue, unf;
    CK(cnt.resize(K + 1)); CK(off.resize(K + 1)); CK(cursor.resize(K + 1)); CK(list.resize(3 * (size_t)t));
    CK(bad.resize(K)); CK(has_nm.resize(K)); CK(issue.resize(K)); CK(unf.resize(K));
    CK(cudaMemsetAsync(cnt.p, 0, (K + 1) * sizeof(unsigned), ctx->s));
    CK(cudaMemsetAsync(cursor.p, 0, (K + 1) * sizeof(unsigned), ctx->s));
    CK(cudaMemsetAsync(has_nm.p, 0, K, ctx->s));
    CK(cudaMemsetAsync(unf.p, 0, K, ctx->s));
    CK(launch_dual_incidence(dt.p, t, cnt.p, nullptr, nullptr, nullptr, false, ctx->s));
    CK(exclusive_scan_u32(cnt.p, off.p, K + 1, nullptr, ctx->scratch, ctx->s));
    CK(launch_dual_incidence(dt.p, t, nullptr, off.p, cursor.p, list.p, true, ctx->s));
    CK(launch_manifold_checks(dt.p, off.p, list.p, K, ctx->edge_int.p, ne, ctx->label.p, nv, ctx->perm.p,
                              ctx->vf_row.p, ctx->vf_face.p, ctx->tri.p, ctx->row.p, ctx->size.p, bad.p, has_nm.p,
                              issue.p, unf.p, ctx->s));
    std::vector<unsigned char> h_issue(K), h_unf(K);
    std::vector<int> h_size(K);
    CK(cudaMemcpyAsync(h_issue.data(), issue.p, K, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(h_unf.data(), unf.p, K, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(h_size.data(), ctx->size.p, K * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    int issues = 0;
    for (int c = 0; c < K; c++) issues += h_issue[c];
    if (issues == 0) return ACVD_OK;

    // the clustering in vertex ids
    std::vector<int> lab(nv);
    CK(ctx->label_orig.resize(nv));
    CK(launch_gather_i32(ctx->label.p, ctx->inv.p, nv, ctx->label_orig.p, ctx->s));
    CK(cudaMemcpyAsync(lab.data(), ctx->label_orig.p, nv * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    // ClusterItems of the clusters with issues, in increasing item id (:175-200)
    std::vector<std::vector<int>> items(K);
    for (int64_t i = 0; i < nv; i++) {
        const int c = lab[i];
        if (c >= 0 && c < K && h_issue[c]) items[c].push_back((int)i);
    }
    // IsClusterFreezed: all but the clusters with issues and their neighbours (:171-174, :236-240)
    std::vector<unsigned char> frozen(K, 1);
    for (int c = 0; c < K; c++)
        if (h_issue[c] || h_unf[c]) frozen[c] = 0;
    std::vector<int> sz(h_size.begin(), h_size.end());
    // vtkIdList::DeleteId: the list's last id takes the freed slot
    auto drop = [&](int c, int item) {
        sz[c]--;
        if (c < K && h_issue[c]) {
            std::vector<int>& v = items[c];
            auto at = std::find(v.begin(), v.end(), item);
            *at = v.back();
            v.pop_back();
        }
    };
    int k_now = K;
    for (int c = 0; c < K; c++) {
        if (!h_issue[c]) continue;
        const int nc = k_now++;          // the new cluster, unfrozen (:257-269)
        frozen.push_back(0);
        sz.push_back(0);
        if (items[c].size() > 1) {
            const int it = items[c][0];
            lab[it] = nc;
            drop(c, it);
            sz[nc] = 1;
            continue;
        }
        // a single item: take the first neighbour item whose cluster has more than one (:285-304)
        const int it = items[c][0];
        int j = 0, rr[2] = {0, 0};
        CK(cudaMemcpy(&j, ctx->inv.p + it, sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rr, ctx->row.p + j, 2 * sizeof(int), cudaMemcpyDeviceToHost));
        std::vector<int> ring(rr[1] - rr[0]);
        if (!ring.empty()) {
            CK(cudaMemcpy(ring.data(), ctx->col.p + rr[0], ring.size() * sizeof(int), cudaMemcpyDeviceToHost));
            for (int& q : ring) CK(cudaMemcpy(&q, ctx->perm.p + q, sizeof(int), cudaMemcpyDeviceToHost));
        }
        bool found = false;
        for (int nb : ring) {
            // a cluster added in this pass holds one item; labels >= K are unassigned
            // items, which the reference never meets here (MinimizeEnergy fills holes)
            const int ncl = lab[nb];
            if (ncl < 0 || ncl >= K) continue;
            if (sz[ncl] > 1) {
                lab[nb] = nc;
                drop(ncl, nb);
                sz[nc] = 1;
                found = true;
                break;
            }
        }
        if (!found) {                    // no freeable neighbour: the new cluster is cancelled (:336-347)
            k_now--;
            frozen.pop_back();
            sz.pop_back();
        }
    }
    // the reference's metric stays in its constrained state after the first run
    ctx->unconstrained = 0;
    if ((r = acvd_set_labels(ctx, k_now, lab.data()))) return r;
    if ((r = acvd_set_frozen_clusters(ctx, frozen.data()))) return r;
    *n_issues = issues;
    *n_clusters = k_now;
    return ACVD_OK;
}

// vtkDiscreteRemeshing::FixMeshBoundaries (DiscreteRemeshing/vtkDiscreteRemeshing.h:426-579)
// for the current clustering.  The device lists the input boundary edges (one face)
// with their endpoints, clusters, valences and points; the host replays the three
// passes over that list in the reference's order.  New output vertices are numbered
// from K; their coordinates are float-rounded as the output's float vtkPoints stores
// them.  Call with NULL buffers to get the counts.
extern "C" int acvd_fix_mesh_boundaries(acvd_ctx* ctx, double* new_points, int64_t* n_new_points, int32_t* new_faces,
                                        int64_t* n_new_faces) {
    if (!ctx || !n_new_points || !n_new_faces) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_fix_mesh_boundaries needs a clustering");
    CK(cudaSetDevice(ctx->opts.device));
    const int64_t nv = ctx->nV, ne = ctx->nE;
    const int K = ctx->K;
    DBuf<uint32_t> flag, pos;
    DBuf<int> ids;
    DBuf<BoundaryEdge> bedges;
    CK(flag.resize(ne + 1));
    CK(pos.resize(ne + 1));
    CK(ctx->dtmp.resize(2));
    uint32_t* total = (uint32_t*)ctx->dtmp.p;
    CK(launch_boundary_edge_flags(ctx->edge_v.p, ne, ctx->vf_row.p, ctx->vf_face.p, ctx->tri.p, flag.p, ctx->s));
    CK(exclusive_scan_u32(flag.p, pos.p, ne, total, ctx->scratch, ctx->s));
    uint32_t nb = 0;
    CK(cudaMemcpyAsync(&nb, total, sizeof nb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    std::vector<BoundaryEdge> be(nb);
    if (nb) {
        CK(ids.resize(nb));
        CK(bedges.resize(nb));
        CK(launch_compact(flag.p, pos.p, ne, ids.p, ctx->s));
        CK(ctx->label_orig.resize(nv));
        CK(launch_gather_i32(ctx->label.p, ctx->inv.p, nv, ctx->label_orig.p, ctx->s));
        CK(launch_boundary_gather(ids.p, nb, ctx->edge_v.p, ctx->label_orig.p, ctx->inv.p, ctx->row.p, ctx->xyz.p,
                                  bedges.p, ctx->s));
        CK(cudaMemcpyAsync(be.data(), bedges.p, nb * sizeof(BoundaryEdge), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    // per vertex, its boundary edges (list positions) in ring order = increasing edge id
    std::vector<std::pair<int, int>> vb;   // (vertex, position)
    vb.reserve(2 * (size_t)nb);
    for (uint32_t b = 0; b < nb; b++) {
        vb.push_back({be[b].v[0], (int)b});
        vb.push_back({be[b].v[1], (int)b});
    }
    std::stable_sort(vb.begin(), vb.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
        return x.first < y.first;
    });
    auto ring_of = [&](int v, size_t& lo, size_t& hi) {
        lo = std::lower_bound(vb.begin(), vb.end(), std::make_pair(v, INT32_MIN)) - vb.begin();
        hi = lo;
        while (hi < vb.size() && vb[hi].first == v) hi++;
    };
    std::vector<int> np(nb, -2);   // EdgesNewPoint
    std::vector<double> pts;
    std::vector<int32_t> faces;
    int n_pts = 0;
    // pass 1: a new vertex and face on every boundary edge between two clusters (:437-465)
    for (uint32_t b = 0; b < nb; b++) {
        const int c1 = be[b].c[0], c2 = be[b].c[1];
        if (c1 == c2) continue;
        for (int q = 0; q < 3; q++)
            pts.push_back((double)(float)(0.5 * (be[b].p1[q] + be[b].p2[q])));
        np[b] = K + n_pts++;
        faces.insert(faces.end(), {np[b], c1, c2});
    }
    // pass 2: every run of boundary edges inside one cluster joins the new vertices
    // at its ends (:467-540)
    std::vector<int> elist;
    for (uint32_t b0 = 0; b0 < nb; b0++) {
        if (np[b0] >= 0) continue;
        const int cluster = be[b0].c[0];
        std::vector<int> queue{(int)b0};
        size_t head = 0;
        elist.clear();
        while (head < queue.size()) {
            const int b = queue[head++];
            if (np[b] == -2) {
                np[b] = -1;
                for (int s = 0; s < 2; s++) {
                    size_t lo, hi;
                    ring_of(be[b].v[s], lo, hi);
                    for (size_t q = lo; q < hi; q++) queue.push_back(vb[q].second);
                }
            } else if (np[b] >= 0) {
                if (std::find(elist.begin(), elist.end(), b) == elist.end()) elist.push_back(b);
            }
        }
        if (elist.size() >= 2) faces.insert(faces.end(), {cluster, np[elist[0]], np[elist[1]]});
    }
    // pass 3: vertices between two new vertices (:542-565).  GetNumberOfBoundaries
    // (Common/vtkSurfaceBase.cxx:939-949) counts the boundary edges among the edges
    // numbered 0 .. valence-1 of the whole mesh, not of the vertex's ring; it is > 0
    // exactly when the valence reaches one past the second boundary edge's number.
    const int64_t need = nb >= 2 ? (int64_t)be[1].edge + 1 : INT64_MAX;
    std::vector<int> verts;
    for (auto& x : vb) if (verts.empty() || verts.back() != x.first) verts.push_back(x.first);
    std::vector<int> nl;
    for (int v : verts) {
        size_t lo, hi;
        ring_of(v, lo, hi);
        const uint32_t b = (uint32_t)vb[lo].second;
        const int deg = be[b].v[0] == v ? be[b].deg[0] : be[b].deg[1];
        const int cl = be[b].v[0] == v ? be[b].c[0] : be[b].c[1];
        if (deg < need) continue;
        nl.clear();
        for (size_t q = lo; q < hi; q++) {
            const int p = np[vb[q].second];
            if (p >= 0 && std::find(nl.begin(), nl.end(), p) == nl.end()) nl.push_back(p);
        }
        if (nl.size() > 1) faces.insert(faces.end(), {cl, nl[0], nl[1]});
    }
    const int64_t nfaces = (int64_t)faces.size() / 3;
    if (new_points && n_pts) {
        if (*n_new_points < n_pts) return fail(ctx, ACVD_ERR_ARG, "acvd_fix_mesh_boundaries: new_points too small");
        std::memcpy(new_points, pts.data(), pts.size() * sizeof(double));
    }
    if (new_faces && nfaces) {
        if (*n_new_faces < nfaces) return fail(ctx, ACVD_ERR_ARG, "acvd_fix_mesh_boundaries: new_faces too small");
        std::memcpy(new_faces, faces.data(), faces.size() * sizeof(int32_t));
    }
    *n_new_points = n_pts;
    *n_new_faces = nfaces;
    return ACVD_OK;
}

// Self-check of the device waits' limit (failure detection without a fault): the
// persistent kernel's grid barrier, with one of two blocks never arriving.
extern "C" int acvd_check_wait_limit(acvd_ctx* ctx, int64_t max_spins, int32_t* gave_up) {
    if (!ctx || !gave_up || max_spins <= 0 || max_spins > (1ll << 24))
        return fail(ctx, ACVD_ERR_ARG, "acvd_check_wait_limit: max_spins outside (0, 2^24]");
    CK(cudaSetDevice(ctx->opts.device));
    DBuf<GridBar> bar;
    CK(bar.resize(1));
    CK(cudaMemsetAsync(bar.p, 0, sizeof(GridBar), ctx->s));
    CK(launch_barrier_wait_limit(bar.p, max_spins, ctx->s));
    GridBar hb;
    CK(cudaMemcpyAsync(&hb, bar.p, sizeof hb, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    *gave_up = hb.err ? 1 : 0;
    return ACVD_OK;
}

extern "C" int acvd_get_dual_mesh(acvd_ctx* ctx, int32_t* tris, int64_t* n_tris) {
    if (!ctx || !n_tris) return ACVD_ERR_ARG;
    if (!ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "no labels");
    CK(cudaSetDevice(ctx->opts.device));
    DBuf<int> out;
    int64_t t = 0;
    const int r = build_dual(ctx, out, &t);
    if (r) return r;
    *n_tris = t;
    if (tris && t) {
        CK(cudaMemcpyAsync(tris, out.p, 3 * (size_t)t * sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
    }
    return ACVD_OK;
}

// ---------------------------------------------------------------------------
// adjoint (fixed clustering)
// ---------------------------------------------------------------------------
namespace acvd {
cudaError_t adjoint_run(const AdjState& a, int metric, int level, double thr, double ratio, double gE,
                        const double* dgE, const double* gC, const uint32_t* sorted, const uint32_t* off,
                        const uint32_t* cnt, double* wsum, double* cent, double* gx, double* grho, cudaStream_t s,
                        Scratch& scratch);
}  // namespace acvd

// The adjoint's work on the context's stream.  g_energy / d_g_energy: the total
// energy's cotangent as a host value or a device scalar (d_g_energy wins when given);
// energy: host output, d_energy: device output.  No host synchronisation.
static int adjoint_enqueue(acvd_ctx* ctx, const double* xyz, const double* rho, double gradation, double g_energy,
                           const double* d_g_energy, const double* g_centroids, double* energy, double* d_energy,
                           double* cluster_energies, double* centroids, double* grad_xyz, double* grad_rho) {
    CK(cudaSetDevice(ctx->opts.device));
    const int64_t nv = ctx->nV, nf = ctx->nF;
    const int K = ctx->K;
    // items sorted by cluster (fixed clustering), in original vertex ids
    CK(ctx->label_orig.resize(nv));
    CK(launch_gather_i32(ctx->label.p, ctx->inv.p, nv, ctx->label_orig.p, ctx->s));
    DevState st = ctx->state();
    st.label = ctx->label_orig.p;
    CK(ctx->wk_a.resize(nv)); CK(ctx->wk_b.resize(nv)); CK(ctx->wk_c.resize(nv)); CK(ctx->wk_d.resize(nv));
    CK(ctx->wk_cnt.resize(K + 1)); CK(ctx->wk_off.resize(K + 1));
    CK(cudaMemsetAsync(ctx->wk_cnt.p, 0, (K + 1) * sizeof(uint32_t), ctx->s));
    CK(launch_cluster_keys(st, ctx->wk_a.p, ctx->wk_b.p, ctx->wk_cnt.p, ctx->s));
    CK(radix_sort_pairs(ctx->wk_a.p, ctx->wk_b.p, ctx->wk_c.p, ctx->wk_d.p, nv, bits_for((uint64_t)K), ctx->scratch,
                        ctx->s));
    CK(exclusive_scan_u32(ctx->wk_cnt.p, ctx->wk_off.p, K + 1, nullptr, ctx->scratch, ctx->s));
    CK(ctx->adj_work.resize(adjoint_bytes(nv, nf, K) + 64));
    AdjState a = adjoint_state(ctx->adj_work.p, nv, nf, K);
    a.x = xyz;
    a.rho = rho;
    a.grad = gradation;
    a.tri = ctx->tri.p;
    a.label = ctx->label_orig.p;
    a.vf_row = ctx->vf_row.p;
    a.vf_face = ctx->vf_face.p;
    CK(ctx->dtmp.resize(4));
    const double ratio = ctx->metric == kQEM ? 10000.0 : 100000.0;
    CK(adjoint_run(a, ctx->metric, ctx->level, 1e-3, ratio, g_energy, d_g_energy, g_centroids, ctx->wk_b.p,
                   ctx->wk_off.p, ctx->wk_cnt.p, ctx->dtmp.p, centroids, grad_xyz, grad_rho, ctx->s, ctx->scratch));
    if (energy || d_energy) {
        CK(sum_f64(a.ek, K, ctx->dtmp.p + 1, ctx->scratch, ctx->s));
        if (d_energy) CK(cudaMemcpyAsync(d_energy, ctx->dtmp.p + 1, sizeof(double), cudaMemcpyDeviceToDevice, ctx->s));
        if (energy) CK(cudaMemcpyAsync(energy, ctx->dtmp.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    }
    if (cluster_energies)
        CK(cudaMemcpyAsync(cluster_energies, a.ek, K * sizeof(double), cudaMemcpyDeviceToDevice, ctx->s));
    return ACVD_OK;
}

static int adjoint_check(acvd_ctx* ctx, const double* xyz) {
    if (!ctx) return ACVD_ERR_ARG;
    if (!ctx->ready_metric || !ctx->ready_labels) return fail(ctx, ACVD_ERR_ARG, "acvd_adjoint needs metric and labels");
    if (!xyz) return fail(ctx, ACVD_ERR_ARG, "acvd_adjoint: positions required");
    if (ctx->metric == kAniso) return fail(ctx, ACVD_ERR_UNSUPPORTED, "adjoint of the anisotropic metric not built");
    return ACVD_OK;
}

extern "C" int acvd_adjoint(acvd_ctx* ctx, const double* xyz, const double* rho, double gradation, double g_energy,
                            const double* g_centroids, double* energy, double* cluster_energies, double* centroids,
                            double* grad_xyz, double* grad_rho) {
    int r = adjoint_check(ctx, xyz);
    if (r) return r;
    r = adjoint_enqueue(ctx, xyz, rho, gradation, g_energy, nullptr, g_centroids, energy, nullptr, cluster_energies,
                        centroids, grad_xyz, grad_rho);
    if (r) return r;
    CK(cudaStreamSynchronize(ctx->s));
    return ACVD_OK;
}

extern "C" int acvd_adjoint_on_stream(acvd_ctx* ctx, void* stream, const double* xyz, const double* rho,
                                      double gradation, const double* d_g_energy, const double* g_centroids,
                                      double* d_energy, double* cluster_energies, double* centroids,
                                      double* grad_xyz, double* grad_rho) {
    int r = adjoint_check(ctx, xyz);
    if (r) return r;
    CK(cudaSetDevice(ctx->opts.device));
    if (!ctx->adj_ev_in) {
        CK(cudaEventCreateWithFlags(&ctx->adj_ev_in, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->adj_ev_out, cudaEventDisableTiming));
    }
    cudaStream_t caller = (cudaStream_t)stream;
    // the caller's earlier work (the inputs) before the context's; the caller's later
    // work after the outputs -- ordering on the device, no host wait
    CK(cudaEventRecord(ctx->adj_ev_in, caller));
    CK(cudaStreamWaitEvent(ctx->s, ctx->adj_ev_in, 0));
    r = adjoint_enqueue(ctx, xyz, rho, gradation, 0.0, d_g_energy, g_centroids, nullptr, d_energy, cluster_energies,
                        centroids, grad_xyz, grad_rho);
    if (r) return r;
    CK(cudaEventRecord(ctx->adj_ev_out, ctx->s));
    CK(cudaStreamWaitEvent(caller, ctx->adj_ev_out, 0));
    return ACVD_OK;
}

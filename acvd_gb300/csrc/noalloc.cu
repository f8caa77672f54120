// Boundary edges of a clustering with no device allocation.
//
// The same result as acvd_get_boundary_edges (edge ids whose two endpoints
// carry different labels, increasing), computed from device buffers the caller
// already holds and enqueued on the caller's stream.  The boundary test is
// fused into the scan: one kernel counts boundary edges per 2048-edge tile, the
// tile counts are scanned, and a second kernel recomputes the test, scans
// within its tile and writes the ids.  The only scratch is the tile counts and
// the scan's own partial sums; they live in a fixed file-scope device array.
#include <mutex>

#include "../../include/acvd_gpu.h"
#include "common.cuh"
#include "primitives.cuh"

// 256 KiB: tile counts (one word per 2048 edges) plus the scan's partial sums
// for the largest accepted input.  Every word a call reads is written by the
// same call first, so nothing has to start at zero.
static constexpr size_t kNoAllocScratchWords = 65536;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

namespace acvd {
namespace {

constexpr int kNaThreads = 1024;
constexpr int64_t kNaTile = 2 * kNaThreads;
constexpr int kNaMaxDevices = 64;

std::mutex g_na_mu;
uint32_t* g_na_ptr[kNaMaxDevices] = {};

__device__ __forceinline__ uint32_t na_flag(const int32_t* __restrict__ ev, const int32_t* __restrict__ label,
                                            int64_t e, int64_t ne) {
    if (e >= ne) return 0u;
    return label[ev[2 * e]] != label[ev[2 * e + 1]] ? 1u : 0u;
}

__global__ void __launch_bounds__(kNaThreads) na_count_kernel(const int32_t* __restrict__ ev, int64_t ne,
                                                              const int32_t* __restrict__ label,
                                                              uint32_t* __restrict__ tile_count) {
    __shared__ uint32_t wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t e0 = (int64_t)blockIdx.x * kNaTile + 2 * tid;
    const uint32_t c = __reduce_add_sync(kFull, na_flag(ev, label, e0, ne) + na_flag(ev, label, e0 + 1, ne));
    if (lane == 0) wsum[wid] = c;
    __syncthreads();
    if (wid == 0) {
        const uint32_t t = __reduce_add_sync(kFull, wsum[lane]);
        if (lane == 0) tile_count[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kNaThreads) na_compact_kernel(const int32_t* __restrict__ ev, int64_t ne,
                                                                const int32_t* __restrict__ label,
                                                                const uint32_t* __restrict__ tile_off,
                                                                int32_t* __restrict__ ids,
                                                                uint32_t* __restrict__ count) {
    __shared__ uint32_t wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t e0 = (int64_t)blockIdx.x * kNaTile + 2 * tid;
    const uint32_t a = na_flag(ev, label, e0, ne), b = na_flag(ev, label, e0 + 1, ne);
    const uint32_t pair = a + b;
    uint32_t incl = pair;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = wsum[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += t;
        }
        wsum[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t at = tile_off[blockIdx.x] + incl - pair + wsum[wid];
    if (a) ids[at] = (int32_t)e0;
    if (b) ids[at + a] = (int32_t)(e0 + 1);
    if (blockIdx.x == gridDim.x - 1 && tid == kNaThreads - 1) *count = at + pair;
}

// Per-device address of the scratch array, looked up once with that device current
// and kept for the process (stale after a cudaDeviceReset of that device).
int na_scratch(uint32_t** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return ACVD_ERR_CUDA;
    if (dev < 0 || dev >= kNaMaxDevices) return ACVD_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return ACVD_ERR_CUDA;
        g_na_ptr[dev] = (uint32_t*)p;
    }
    *out = g_na_ptr[dev];
    return ACVD_OK;
}

}  // namespace
}  // namespace acvd

extern "C" int acvd_boundary_edges_noalloc(const int32_t* d_edge_v, int64_t n_edges, const int32_t* d_labels,
                                           int32_t* d_ids, uint32_t* d_count, void* stream) {
    using namespace acvd;
    if (n_edges < 0 || !d_count) return ACVD_ERR_ARG;
    if (n_edges > 0 && (!d_edge_v || !d_labels || !d_ids)) return ACVD_ERR_ARG;
    if (n_edges > ACVD_NOALLOC_MAX_EDGES) return ACVD_ERR_UNSUPPORTED;
    static_assert((ACVD_NOALLOC_MAX_EDGES + kNaTile - 1) / kNaTile + 18 <= kNoAllocScratchWords,
                  "scratch array too small for the largest accepted input");
    uint32_t* scratch = nullptr;
    const int rc = na_scratch(&scratch);
    if (rc != ACVD_OK) return rc;
    const int64_t nb = n_edges > 0 ? (n_edges + kNaTile - 1) / kNaTile : 1;
    const size_t need = (size_t)nb + scan_scratch_need(nb);
    if (need > kNoAllocScratchWords) return ACVD_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* tile = scratch;
    ++g_launches;
    na_count_kernel<<<(unsigned)nb, kNaThreads, 0, s>>>(d_edge_v, n_edges, d_labels, tile);
    if (cudaGetLastError() != cudaSuccess) return ACVD_ERR_CUDA;
    if (exclusive_scan_u32_raw(tile, tile, nb, scratch + nb, kNoAllocScratchWords - (size_t)nb, s) != cudaSuccess)
        return ACVD_ERR_CUDA;
    ++g_launches;
    na_compact_kernel<<<(unsigned)nb, kNaThreads, 0, s>>>(d_edge_v, n_edges, d_labels, tile, d_ids, d_count);
    if (cudaGetLastError() != cudaSuccess) return ACVD_ERR_CUDA;
    return ACVD_OK;
}

// Device-wide primitives: exclusive scan, deterministic FP64 sum, stable radix sort.
#include "primitives.cuh"
#include "common.cuh"

#include <algorithm>

namespace acvd {

long long g_launches = 0;

cudaError_t Scratch::reserve(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    const size_t want = std::max(need, bytes * 2);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) bytes = want;
    return e;
}

Scratch::~Scratch() {
    if (ptr) cudaFree(ptr);
}

// ---------------------------------------------------------------------------
// exclusive scan of uint32 (1024 threads x 2 elements per block)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 2 * kScanThreads;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// `in` and `out` may be the same array (in-place scans): each thread reads its
// own pair before the block's first barrier and writes it after the last, so
// neither pointer is declared __restrict__.
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                                                 uint32_t* __restrict__ block_sums) {
    __shared__ uint32_t wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanTile + 2 * tid;
    const uint32_t a = base < n ? in[base] : 0u;
    const uint32_t b = base + 1 < n ? in[base + 1] : 0u;
    const uint32_t pair = a + b;
    const uint32_t incl = warp_incl_scan(pair, lane);
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = wsum[lane];
        const uint32_t wi = warp_incl_scan(w, lane);
        wsum[lane] = wi - w;
        if (lane == 31 && block_sums) block_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    const uint32_t excl = incl - pair + wsum[wid];
    if (base < n) out[base] = excl;
    if (base + 1 < n) out[base + 1] = excl + a;
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, int64_t n, const uint32_t* __restrict__ offs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offs[i / kScanTile];
}

// total = last exclusive prefix + last input (saved before an in-place scan)
__global__ void scan_total_kernel(const uint32_t* last_in, const uint32_t* out, int64_t n, uint32_t* total) {
    if (n == 0) { *total = 0; return; }
    *total = out[n - 1] + last_in[0];
}

static size_t scan_scratch_words(int64_t n) {
    size_t w = 0;
    while (n > kScanTile) {
        n = (n + kScanTile - 1) / kScanTile;
        w += (size_t)n + 1;
    }
    return w + 1;
}

static cudaError_t scan_rec(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        ++g_launches;
        scan_tile_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
        return cudaGetLastError();
    }
    uint32_t* sums = scratch;
    ++g_launches;
    scan_tile_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums);
    cudaError_t e = scan_rec(sums, sums, nb, scratch + nb + 1, s);
    if (e != cudaSuccess) return e;
    ++g_launches;
    scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums);
    return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev,
                               Scratch& scratch, cudaStream_t s) {
    // the total must be read before `out` overwrites `in` (in-place scan)
    const size_t words = scan_scratch_words(n) + 1;
    cudaError_t e = scratch.reserve(words * sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    uint32_t* sc = (uint32_t*)scratch.ptr;
    uint32_t* last = sc + words - 1;
    if (total_dev && n > 0) {
        e = cudaMemcpyAsync(last, in + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    e = scan_rec(in, out, n, sc, s);
    if (e != cudaSuccess) return e;
    if (total_dev) {
        ++g_launches;
        scan_total_kernel<<<1, 1, 0, s>>>(last, out, n, total_dev);
        e = cudaGetLastError();
    }
    return e;
}

size_t scan_scratch_need(int64_t n) { return scan_scratch_words(n); }

cudaError_t exclusive_scan_u32_raw(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch,
                                   size_t scratch_words, cudaStream_t s) {
    if (scratch_words < scan_scratch_words(n)) return cudaErrorInvalidValue;
    return scan_rec(in, out, n, scratch, s);
}

// ---------------------------------------------------------------------------
// deterministic FP64 sum: fixed-shape tree (256-thread blocks, 8 values/thread)
// ---------------------------------------------------------------------------

__global__ void sum_f64_kernel(const double* __restrict__ in, int64_t n, double* __restrict__ out) {
    sum_f64_chunk(in, n, blockIdx.x, out);
}

cudaError_t sum_f64(const double* in, int64_t n, double* out_dev, Scratch& scratch, cudaStream_t s) {
    const int64_t per = (int64_t)kSumThreads * kSumPer;
    int64_t nb = (n + per - 1) / per;
    if (nb < 1) nb = 1;
    const int64_t nb2 = (nb + per - 1) / per;
    cudaError_t e = scratch.reserve((size_t)(nb + nb2 + 2) * sizeof(double));
    if (e != cudaSuccess) return e;
    double* a = (double*)scratch.ptr;
    double* b = a + nb + 1;
    ++g_launches;
    sum_f64_kernel<<<(unsigned)nb, kSumThreads, 0, s>>>(in, n, a);
    const double* cur = a;
    int64_t m = nb;
    double* dst = b;
    double* other = a;
    while (m > 1) {
        const int64_t mb = (m + per - 1) / per;
        ++g_launches;
        sum_f64_kernel<<<(unsigned)mb, kSumThreads, 0, s>>>(cur, m, dst);
        cur = dst;
        m = mb;
        double* t = dst; dst = other; other = t;
    }
    e = cudaMemcpyAsync(out_dev, cur, sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// stable LSD radix sort, 8 bits per pass.  Each warp owns a tile of kSortTile
// consecutive elements and walks it in order, 32 at a time; ranks inside a
// 32-element chunk come from __match_any_sync, so the scatter is stable.
// counts are laid out digit-major: counts[digit * ntiles + tile].
// ---------------------------------------------------------------------------
constexpr int kSortWarps = 8;
constexpr int kSortTile = 1024;

__global__ void __launch_bounds__(kSortWarps * 32) radix_hist_kernel(const uint32_t* __restrict__ keys, int64_t n,
                                                                     int shift, int64_t ntiles,
                                                                     uint32_t* __restrict__ counts) {
    __shared__ uint32_t hist[kSortWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t tile = (int64_t)blockIdx.x * kSortWarps + w;
    for (int d = lane; d < 256; d += 32) hist[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        const int64_t base = tile * kSortTile;
        for (int c = 0; c < kSortTile; c += 32) {
            const int64_t i = base + c + lane;
            if (i < n) atomicAdd(&hist[w][(keys[i] >> shift) & 255u], 1u);
        }
        __syncwarp();
        for (int d = lane; d < 256; d += 32) counts[(int64_t)d * ntiles + tile] = hist[w][d];
    }
}

__global__ void __launch_bounds__(kSortWarps * 32) radix_scatter_kernel(
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t* __restrict__ okeys,
    uint32_t* __restrict__ ovals, int64_t n, int shift, int64_t ntiles, const uint32_t* __restrict__ offsets) {
    __shared__ uint32_t run[kSortWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t tile = (int64_t)blockIdx.x * kSortWarps + w;
    if (tile >= ntiles) return;
    for (int d = lane; d < 256; d += 32) run[w][d] = offsets[(int64_t)d * ntiles + tile];
    __syncwarp();
    const int64_t base = tile * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int c = 0; c < kSortTile; c += 32) {
        const int64_t i = base + c + lane;
        const bool valid = i < n;
        const unsigned active = __ballot_sync(kFull, valid);
        if (active == 0) break;
        uint32_t k = 0, v = 0, d = 256u + lane;   // invalid lanes get unique dummy digits
        if (valid) { k = keys[i]; v = vals[i]; d = (k >> shift) & 255u; }
        const unsigned peers = __match_any_sync(kFull, d);
        const uint32_t rank = __popc(peers & lt);
        uint32_t pos = 0;
        if (valid) pos = run[w][d] + rank;
        __syncwarp();
        if (valid) {
            okeys[pos] = k;
            ovals[pos] = v;
            const int leader = __ffs(peers) - 1;
            if (lane == leader) run[w][d] += __popc(peers);
        }
        __syncwarp();
    }
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* tmp_keys, uint32_t* tmp_vals, int64_t n,
                             int key_bits, Scratch& scratch, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    const int64_t ncounts = 256 * ntiles;
    const size_t scan_words = scan_scratch_words(ncounts) + 2;
    cudaError_t e = scratch.reserve((size_t)(ncounts + scan_words) * sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    uint32_t* counts = (uint32_t*)scratch.ptr;
    uint32_t* sc = counts + ncounts;
    const unsigned blocks = (unsigned)((ntiles + kSortWarps - 1) / kSortWarps);
    const int passes = (key_bits + 7) / 8;
    uint32_t *ka = keys, *va = vals, *kb = tmp_keys, *vb = tmp_vals;
    for (int p = 0; p < passes; p++) {
        const int shift = 8 * p;
        ++g_launches;
        radix_hist_kernel<<<blocks, kSortWarps * 32, 0, s>>>(ka, n, shift, ntiles, counts);
        e = scan_rec(counts, counts, ncounts, sc, s);
        if (e != cudaSuccess) return e;
        ++g_launches;
        radix_scatter_kernel<<<blocks, kSortWarps * 32, 0, s>>>(ka, va, kb, vb, n, shift, ntiles, counts);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        uint32_t* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        e = cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
    return e;
}

}  // namespace acvd

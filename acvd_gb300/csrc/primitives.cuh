// Device-wide primitives used by the clustering pipeline: exclusive scan,
// deterministic FP64 sums and a stable LSD radix sort of (key, value) pairs.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace acvd {

// Number of kernels launched by this library (host-side count of <<<>>> sites).
extern long long g_launches;

// Scratch for the primitives; grown on demand, owned by the caller's context.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t need);
    ~Scratch();
};

// out[i] = sum_{j<i} in[j] for n uint32 values (in == out allowed).  total may be null.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev,
                               Scratch& scratch, cudaStream_t s);

// Stable sort of (keys, vals) by the low `key_bits` bits of keys.  Results land in
// keys/vals; tmp_keys/tmp_vals are same-sized work buffers.
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* tmp_keys, uint32_t* tmp_vals,
                             int64_t n, int key_bits, Scratch& scratch, cudaStream_t s);

// Scratch words exclusive_scan_u32_raw needs for n values.
size_t scan_scratch_need(int64_t n);

// exclusive_scan_u32 without a total, on caller-provided scratch of
// scratch_words uint32 words (at least scan_scratch_need(n)); allocates nothing.
cudaError_t exclusive_scan_u32_raw(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch,
                                   size_t scratch_words, cudaStream_t s);

// Deterministic sum of n doubles (fixed reduction tree) into *out_dev.
cudaError_t sum_f64(const double* in, int64_t n, double* out_dev, Scratch& scratch, cudaStream_t s);

#ifdef __CUDACC__
// One chunk of the deterministic FP64 sum: 256 threads (the whole block, every
// thread calls it) add values chunk*2048 .. +2047 in a fixed tree; out[chunk]
// receives the chunk's sum.  sum_f64 applies it level by level.
constexpr int kSumThreads = 256;
constexpr int kSumPer = 8;

__device__ __forceinline__ void sum_f64_chunk(const double* in, int64_t n, int64_t chunk, double* out) {
    __shared__ double sh[kSumThreads];
    const int tid = threadIdx.x;
    const int64_t base = chunk * kSumThreads * kSumPer;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < kSumPer; k++) {
        const int64_t i = base + (int64_t)k * kSumThreads + tid;
        if (i < n) acc += in[i];
    }
    __syncthreads();   // a previous chunk of this block is done with sh
    sh[tid] = acc;
    __syncthreads();
    for (int o = kSumThreads / 2; o > 0; o >>= 1) {
        if (tid < o) sh[tid] += sh[tid + o];
        __syncthreads();
    }
    if (tid == 0) out[chunk] = sh[0];
}
#endif

// Number of bits needed to represent values in [0, v].
inline int bits_for(uint64_t v) {
    int b = 1;
    while ((1ull << b) <= v && b < 63) b++;
    return b;
}

}  // namespace acvd

// One-time per-mesh kernels: ring adjacency bitmasks, graph colouring and the
// per-vertex item records (dual areas, weights, quadrics, anisotropic tensors).
#include "primitives.cuh"
#include "state.cuh"

namespace acvd {

// ---------------------------------------------------------------------------
// Ring adjacency: for item i with ring slots p = 0..d-1 (neighbours col[row[i]+p]),
// adj[row[i]+p] has bit q set when neighbour p and neighbour q are themselves
// joined by a mesh edge.  With it the reference's local connectivity test
// (vtkVerticesProcessing.h:168-237: are the same-cluster ring members connected
// through edges among themselves?) becomes a few bit operations.  Rings longer
// than 32 get no mask; the evaluation kernels refuse their moves while the
// connectivity constraint is on.
// ---------------------------------------------------------------------------
__global__ void ring_adjacency_kernel(const int* __restrict__ row, const int* __restrict__ col, int64_t n,
                                      unsigned* __restrict__ adj, int* __restrict__ max_deg) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int d_or = i < n ? row[i + 1] - row[i] : 0;
    const int dmax = __reduce_max_sync(kFull, d_or);   // one atomic per warp
    if ((threadIdx.x & 31) == 0) atomicMax(max_deg, dmax);
    if (i >= n) return;
    const int p0 = row[i], p1 = row[i + 1];
    const int d = p1 - p0;
    if (d > 32) {
        for (int p = p0; p < p1; p++) adj[p] = 0u;
        return;
    }
    for (int p = 0; p < d; p++) {
        const int u = col[p0 + p];
        const int u0 = row[u], u1 = row[u + 1];
        unsigned m = 0u;
        for (int t = u0; t < u1; t++) {
            const int w = col[t];
            for (int q = 0; q < d; q++)
                if (q != p && col[p0 + q] == w) m |= 1u << q;
        }
        adj[p0 + p] = m;
    }
}

cudaError_t launch_ring_adjacency(const int* row, const int* col, int64_t n, unsigned* adj, int* max_deg,
                                  cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    ring_adjacency_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(row, col, n, adj, max_deg);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Jones-Plassmann colouring with hashed priorities (deterministic).  An
// uncoloured item whose priority beats every uncoloured neighbour takes the
// smallest colour unused around it; adjacent items never colour in the same
// round.  Up to 64 colours.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t jp_hash(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// remaining: the counter stripes (the block adds into its own); max_color: the
// largest colour handed out.  Both are updated once per warp.
__global__ void color_round_kernel(const int* __restrict__ row, const int* __restrict__ col, int64_t n,
                                   int* __restrict__ color, unsigned long long* __restrict__ remaining,
                                   int* __restrict__ max_color) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool blocked = false;
    int c = -1;
    if (i < n && color[i] < 0) {
        const uint32_t hi = jp_hash((uint32_t)i);
        const int p0 = row[i], p1 = row[i + 1];
        unsigned long long used = 0ull;
        for (int p = p0; p < p1 && !blocked; p++) {
            const int j = col[p];
            const int cj = color[j];
            if (cj < 0) {
                const uint32_t hj = jp_hash((uint32_t)j);
                if (hj > hi || (hj == hi && j > i)) blocked = true;
            } else if (cj < 64) {
                used |= 1ull << cj;
            }
        }
        if (!blocked) {
            c = used == ~0ull ? 64 : __ffsll((long long)~used) - 1;
            color[i] = c;
        }
    }
    const unsigned nb = __popc(__ballot_sync(kFull, blocked));
    const int cmax = __reduce_max_sync(kFull, c);
    if ((threadIdx.x & 31) == 0) {
        if (nb) atomicAdd(remaining + (blockIdx.x & (kStripes - 1)) * kNumCounters, (unsigned long long)nb);
        if (cmax >= 0) atomicMax(max_color, cmax);
    }
}

cudaError_t launch_color_round(const int* row, const int* col, int64_t n, int* color,
                               unsigned long long* remaining, int* max_color, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    color_round_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(row, col, n, color, remaining, max_color);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Face geometry in FP64: area by the side-length form the reference uses
// (Common/vtkSurface.cxx:1283) and the unit normal that defines the face's
// plane quadric (Common/vtkQuadricTools.cxx:56-79).
// ---------------------------------------------------------------------------
__global__ void face_geometry_kernel(const double* __restrict__ xyz, const int* __restrict__ tri, int64_t nf,
                                     double* __restrict__ farea, double* __restrict__ fnorm) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int a = tri[3 * f], b = tri[3 * f + 1], c = tri[3 * f + 2];
    const double p1[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
    const double p2[3] = {xyz[3 * b], xyz[3 * b + 1], xyz[3 * b + 2]};
    const double p3[3] = {xyz[3 * c], xyz[3 * c + 1], xyz[3 * c + 2]};
    double d12 = 0, d23 = 0, d31 = 0;
    for (int k = 0; k < 3; k++) {
        d12 += (p1[k] - p2[k]) * (p1[k] - p2[k]);
        d23 += (p2[k] - p3[k]) * (p2[k] - p3[k]);
        d31 += (p3[k] - p1[k]) * (p3[k] - p1[k]);
    }
    const double t = d12 - d23 + d31;
    farea[f] = 0.25 * sqrt(fabs(4.0 * d12 * d31 - t * t));
    const double e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const double e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    double nx = e1[1] * e2[2] - e1[2] * e2[1];
    double ny = e1[2] * e2[0] - e1[0] * e2[2];
    double nz = e1[0] * e2[1] - e1[1] * e2[0];
    const double len = sqrt(nx * nx + ny * ny + nz * nz);
    if (len > 0.0) { nx /= len; ny /= len; nz /= len; } else { nx = ny = nz = 0.0; }
    fnorm[3 * f] = nx; fnorm[3 * f + 1] = ny; fnorm[3 * f + 2] = nz;
}

cudaError_t launch_face_geometry(const double* xyz, const int* tri, int64_t nf, double* farea, double* fnorm,
                                 cudaStream_t s) {
    if (nf == 0) return cudaSuccess;
    ++g_launches;
    face_geometry_kernel<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(xyz, tri, nf, farea, fnorm);
    return cudaGetLastError();
}

// (vertex, face) pairs in face order; a stable sort by vertex yields every
// vertex's faces in increasing face id.
__global__ void vertex_keys_kernel(const int* __restrict__ tri, int64_t nf, uint32_t* __restrict__ keys,
                                   uint32_t* __restrict__ vals) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 3 * nf) return;
    keys[j] = (uint32_t)tri[j];
    vals[j] = (uint32_t)(j / 3);
}

cudaError_t launch_vertex_keys(const int* tri, int64_t nf, uint32_t* keys, uint32_t* vals, cudaStream_t s) {
    if (nf == 0) return cudaSuccess;
    ++g_launches;
    vertex_keys_kernel<<<(unsigned)((3 * nf + 255) / 256), 256, 0, s>>>(tri, nf, keys, vals);
    return cudaGetLastError();
}

// Segment offsets of sorted keys in [0, nkeys): off[c] = first position whose key
// is >= c, off[nkeys] = n.  Thread j writes the offsets of the keys from the
// previous element's key (exclusive) to its own (inclusive); thread n closes the
// tail.  Every offset is written exactly once; no atomics.
__global__ void segment_offsets_kernel(const uint32_t* __restrict__ keys, int64_t n, uint32_t nkeys,
                                       uint32_t* __restrict__ off) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > n) return;
    const uint32_t lo = j == 0 ? 0u : keys[j - 1] + 1u;
    const uint32_t hi = j == n ? nkeys : keys[j];
    for (uint32_t c = lo; c <= hi && c <= nkeys; c++) off[c] = (uint32_t)j;
}

cudaError_t launch_segment_offsets(const uint32_t* sorted_keys, int64_t n, uint32_t nkeys, uint32_t* off,
                                   cudaStream_t s) {
    ++g_launches;
    segment_offsets_kernel<<<(unsigned)((n + 1 + 255) / 256), 256, 0, s>>>(sorted_keys, n, nkeys, off);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-vertex items, FP64 inside (BuildMetric of the three metric plugins):
// dual area = sum of adjacent face areas / 3 (Common/vtkSurface.cxx:1342-1359),
// weight = area * indicator^gradation (when an indicator is given), quadric
// A = sum n n^T over adjacent faces.
// ---------------------------------------------------------------------------
__global__ void vertex_items_kernel(int metric, int64_t nv, const uint32_t* __restrict__ vf_row,
                                    const uint32_t* __restrict__ vf_face, const double* __restrict__ farea,
                                    const double* __restrict__ fnorm, const double* __restrict__ indicator,
                                    double gradation, double* __restrict__ wd, double* __restrict__ varea,
                                    float4* __restrict__ qa, float2* __restrict__ qb) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const uint32_t f0 = vf_row[v], f1 = vf_row[v + 1];
    double area = 0.0;
    double A[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t j = f0; j < f1; j++) {
        const uint32_t f = vf_face[j];
        area += farea[f] / 3.0;
        const double nx = fnorm[3 * f], ny = fnorm[3 * f + 1], nz = fnorm[3 * f + 2];
        A[0] += nx * nx; A[1] += nx * ny; A[2] += nx * nz;
        A[3] += ny * ny; A[4] += ny * nz; A[5] += nz * nz;
    }
    double w = area;
    if (indicator) w = area * pow(indicator[v], gradation);
    wd[v] = w;
    varea[v] = area;
    if (metric != kIso) {
        qa[v] = make_float4((float)A[0], (float)A[1], (float)A[2], (float)A[3]);
        qb[v] = make_float2((float)A[4], (float)A[5]);
    }
}

cudaError_t launch_vertex_items(int metric, int64_t nv, const double* xyz, const uint32_t* vf_row,
                                const uint32_t* vf_face, const double* farea, const double* fnorm,
                                const double* indicator, double gradation, double* wd, double* varea,
                                float4* qa, float2* qb, cudaStream_t s) {
    (void)xyz;
    if (nv == 0) return cudaSuccess;
    ++g_launches;
    vertex_items_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, s>>>(metric, nv, vf_row, vf_face, farea, fnorm,
                                                                      indicator, gradation, wd, varea, qa, qb);
    return cudaGetLastError();
}

// Weight clamping to [mean / ratio, mean * ratio] (ClampWeights of the metric
// plugins) and the float32 item records.  Anisotropic tensor:
// area * (d1 d1^T + d2 d2^T) from the principal directions d1 = pd[0..2],
// d2 = pd[3..5], with entry (1,1) built from pd[1]^2 + pd[5]^2 as the reference
// builds it (vtkQuadricAnisotropicMetricForClustering.h:442-446).
// Batched meshes: the mesh of vertex v (vertex offsets v_off[0..nmesh]).
__device__ __forceinline__ int mesh_of(const int64_t* v_off, int nmesh, int64_t v) {
    int lo = 0, hi = nmesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (v_off[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// one block per mesh: fixed-order FP64 sum of the weights of its vertex range
__global__ void mesh_sums_kernel(const double* __restrict__ wd, const int64_t* __restrict__ v_off,
                                 double* __restrict__ out) {
    __shared__ double sh[256];
    const int m = blockIdx.x;
    const int64_t a = v_off[m], b = v_off[m + 1];
    double acc = 0.0;
    for (int64_t v = a + threadIdx.x; v < b; v += 256) acc += wd[v];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[m] = sh[0];
}

cudaError_t launch_mesh_sums(const double* wd, const int64_t* v_off, int nmesh, double* out, cudaStream_t s) {
    if (nmesh == 0) return cudaSuccess;
    ++g_launches;
    mesh_sums_kernel<<<nmesh, 256, 0, s>>>(wd, v_off, out);
    return cudaGetLastError();
}

__global__ void finish_items_kernel(int metric, int64_t nv, const double* __restrict__ xyz,
                                    const double* __restrict__ wd, const double* __restrict__ varea,
                                    const double* __restrict__ wsum, const int64_t* __restrict__ v_off, int nmesh,
                                    double ratio, const float* __restrict__ pd,
                                    float4* __restrict__ xw, float4* __restrict__ ta, float2* __restrict__ tb) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    // the mean is taken over the vertex's own mesh (every mesh of a batch is clamped
    // as if it were clustered alone)
    double mean;
    if (v_off) {
        const int m = mesh_of(v_off, nmesh, v);
        mean = wsum[m] / (double)(v_off[m + 1] - v_off[m]);
    } else {
        mean = *wsum / (double)nv;
    }
    const double lo = mean / ratio, hi = mean * ratio;
    double w = wd[v];
    if (w > hi) w = hi;
    if (w < lo) w = lo;
    xw[v] = make_float4((float)xyz[3 * v], (float)xyz[3 * v + 1], (float)xyz[3 * v + 2], (float)w);
    if (metric == kAniso) {
        const double a = varea[v];
        double P[6];
        for (int j = 0; j < 6; j++) P[j] = (double)pd[6 * v + j];
        const float t0 = (float)(a * P[0] * P[0] + a * P[3] * P[3]);
        const float t1 = (float)(a * P[0] * P[1] + a * P[3] * P[4]);
        const float t2 = (float)(a * P[0] * P[2] + a * P[3] * P[5]);
        const float t3 = (float)(a * P[1] * P[1] + a * P[5] * P[5]);
        const float t4 = (float)(a * P[1] * P[2] + a * P[4] * P[5]);
        const float t5 = (float)(a * P[2] * P[2] + a * P[5] * P[5]);
        ta[v] = make_float4(t0, t1, t2, t3);
        tb[v] = make_float2(t4, t5);
    }
}

cudaError_t launch_finish_items(int metric, int64_t nv, const double* xyz, const double* wd, const double* varea,
                                const double* wsum, const int64_t* v_off, int nmesh, double ratio, const float* pdirs,
                                float4* xw, float4* ta, float2* tb, cudaStream_t s) {
    if (nv == 0) return cudaSuccess;
    ++g_launches;
    finish_items_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, s>>>(metric, nv, xyz, wd, varea, wsum, v_off, nmesh,
                                                                      ratio, pdirs, xw, ta, tb);
    return cudaGetLastError();
}

}  // namespace acvd

namespace acvd {

// ---------------------------------------------------------------------------
// Internal item order.  After colouring, items are renumbered so that every
// colour class is one contiguous range (class by class, increasing original id
// inside a class): perm[t] = original id of internal item t, inv[v] = internal
// id of original vertex v.  The ring CSR is rebuilt in internal ids with each
// ring's order kept, so the per-item streams of a colour step are coalesced.
// ---------------------------------------------------------------------------
__global__ void scatter_inv_kernel(const int* __restrict__ perm, int64_t n, int* __restrict__ inv) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) inv[perm[t]] = (int)t;
}

__global__ void perm_degree_kernel(const int* __restrict__ row, const int* __restrict__ perm, int64_t n,
                                   uint32_t* __restrict__ deg) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const int v = perm[t];
        deg[t] = (uint32_t)(row[v + 1] - row[v]);
    } else if (t == n) {
        deg[n] = 0u;
    }
}

__global__ void perm_ring_kernel(const int* __restrict__ row, const int* __restrict__ col,
                                 const int* __restrict__ perm, const int* __restrict__ inv,
                                 const uint32_t* __restrict__ row_new, int64_t n, int* __restrict__ col_new) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int v = perm[t];
    const int p0 = row[v], p1 = row[v + 1];
    const uint32_t o = row_new[t];
    for (int q = 0; q < p1 - p0; q++) col_new[o + q] = inv[col[p0 + q]];
}

__global__ void map_ids_kernel(const int* __restrict__ in, int64_t m, const int* __restrict__ inv,
                               int* __restrict__ out) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m) out[j] = inv[in[j]];
}

template <typename T>
__global__ void gather_kernel(const T* __restrict__ src, const int* __restrict__ idx, int64_t n,
                              T* __restrict__ dst) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = src[idx[t]];
}

__global__ void iota_kernel(int64_t n, int* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (int)t;
}

// Fixed-width copy of the first 8 ring slots (ring order), -1 padded; slot 7 =
// -2 when the ring has more than 8 neighbours.  The evaluation reads an item's
// neighbours without first reading its CSR bounds.
__global__ void ring8_kernel(const int* __restrict__ row, const int* __restrict__ col, int64_t n,
                             int* __restrict__ ring8) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p0 = row[t], d = row[t + 1] - p0;
    for (int q = 0; q < 8; q++) ring8[8 * t + q] = q < d ? col[p0 + q] : -1;
    if (d > 8) ring8[8 * t + 7] = -2;
}

static inline unsigned grid_of(int64_t n) { return (unsigned)((n + 255) / 256); }

cudaError_t launch_ring8(const int* row, const int* col, int64_t n, int* ring8, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    ring8_kernel<<<grid_of(n), 256, 0, s>>>(row, col, n, ring8);
    return cudaGetLastError();
}

cudaError_t launch_scatter_inv(const int* perm, int64_t n, int* inv, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    scatter_inv_kernel<<<grid_of(n), 256, 0, s>>>(perm, n, inv);
    return cudaGetLastError();
}

cudaError_t launch_perm_degree(const int* row, const int* perm, int64_t n, uint32_t* deg, cudaStream_t s) {
    ++g_launches;
    perm_degree_kernel<<<grid_of(n + 1), 256, 0, s>>>(row, perm, n, deg);
    return cudaGetLastError();
}

cudaError_t launch_perm_ring(const int* row, const int* col, const int* perm, const int* inv, const uint32_t* row_new,
                             int64_t n, int* col_new, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    perm_ring_kernel<<<grid_of(n), 256, 0, s>>>(row, col, perm, inv, row_new, n, col_new);
    return cudaGetLastError();
}

cudaError_t launch_map_ids(const int* in, int64_t m, const int* inv, int* out, cudaStream_t s) {
    if (m == 0) return cudaSuccess;
    ++g_launches;
    map_ids_kernel<<<grid_of(m), 256, 0, s>>>(in, m, inv, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_i32(const int* src, const int* idx, int64_t n, int* dst, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    gather_kernel<int><<<grid_of(n), 256, 0, s>>>(src, idx, n, dst);
    return cudaGetLastError();
}

// Mesh arrays as uploaded: ring offsets non-decreasing, every vertex id (ring
// neighbours, face corners, edge ends) in [0, n).  Counts the violations in *bad,
// before any kernel indexes with those ids.
__global__ void validate_mesh_kernel(const int* __restrict__ row, const int* __restrict__ col, int64_t n,
                                     int64_t ncol, const int* __restrict__ tri, int64_t ntri,
                                     const int* __restrict__ ev, int64_t nev, unsigned* __restrict__ bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned cnt = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride)
        cnt += row[t] > row[t + 1];
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncol; t += stride)
        cnt += (unsigned)col[t] >= (unsigned)n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntri; t += stride)
        cnt += (unsigned)tri[t] >= (unsigned)n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nev; t += stride)
        cnt += (unsigned)ev[t] >= (unsigned)n;
    if (cnt) atomicAdd(bad, cnt);
}

cudaError_t launch_validate_mesh(const int* row, const int* col, int64_t n, int64_t ncol, const int* tri,
                                 int64_t ntri, const int* ev, int64_t nev, unsigned* bad, cudaStream_t s) {
    ++g_launches;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    validate_mesh_kernel<<<4 * sms, 256, 0, s>>>(row, col, n, ncol, tri, ntri, ev, nev, bad);
    return cudaGetLastError();
}

// dst[t] = src[idx[t]] for labels, counting the values outside [0, k] in *bad
__global__ void gather_labels_kernel(const int* __restrict__ src, const int* __restrict__ idx, int64_t n, int k,
                                     int* __restrict__ dst, unsigned* __restrict__ bad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int v = src[idx[t]];
    dst[t] = v;
    if (v < 0 || v > k) atomicAdd(bad, 1u);
}

cudaError_t launch_gather_labels(const int* src, const int* idx, int64_t n, int k, int* dst, unsigned* bad,
                                 cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    gather_labels_kernel<<<grid_of(n), 256, 0, s>>>(src, idx, n, k, dst, bad);
    return cudaGetLastError();
}

// ids were range-checked on the host: -1 or a vertex id
__global__ void anchor_setup_kernel(const int* __restrict__ ids, int n, const int* __restrict__ inv,
                                    const double* __restrict__ xyz, int* __restrict__ item_out,
                                    double* __restrict__ xyz_out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int v = ids[c];
    item_out[c] = v >= 0 ? inv[v] : -1;
    if (xyz_out)
        for (int j = 0; j < 3; j++) xyz_out[3 * (int64_t)c + j] = v >= 0 ? xyz[3 * (int64_t)v + j] : 0.0;
}

cudaError_t launch_anchor_setup(const int* ids, int n, const int* inv, const double* xyz, int* item_out,
                                double* xyz_out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    anchor_setup_kernel<<<grid_of(n), 256, 0, s>>>(ids, n, inv, xyz, item_out, xyz_out);
    return cudaGetLastError();
}

cudaError_t launch_gather_f4(const float4* src, const int* idx, int64_t n, float4* dst, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    gather_kernel<float4><<<grid_of(n), 256, 0, s>>>(src, idx, n, dst);
    return cudaGetLastError();
}

cudaError_t launch_gather_f2(const float2* src, const int* idx, int64_t n, float2* dst, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    gather_kernel<float2><<<grid_of(n), 256, 0, s>>>(src, idx, n, dst);
    return cudaGetLastError();
}

cudaError_t launch_iota(int64_t n, int* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ++g_launches;
    iota_kernel<<<grid_of(n), 256, 0, s>>>(n, out);
    return cudaGetLastError();
}

}  // namespace acvd

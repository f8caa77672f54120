// Manifold checks of vtkDiscreteRemeshing's ForceManifold loop
// (DetectNonManifoldOutputVertices, DiscreteRemeshing/vtkDiscreteRemeshing.h:165-383)
// and the input boundary edges its FixMeshBoundaries walks (:426-579).
//
// vtkSurfaceBase::IsVertexManifold (Common/vtkSurfaceBase.cxx:259-315) is true when
// the vertex has at least two edges, every edge has exactly two faces
// (IsEdgeManifold, vtkSurfaceBase.h:521-528: a boundary edge, an edge without a
// face or an edge with a third face fails) and its faces form a single fan around
// it.  These kernels evaluate the same predicate from face incidence, which does not
// depend on the edge or ring order the reference walks in:
//  * an output (dual) vertex: its incident dual triangles -- each neighbour on
//    exactly two of them, and one cycle through all of them -- plus the
//    cluster-adjacency edges BuildDelaunayTriangulation adds under ForceManifold
//    (:1114-1132): a pair of adjacent clusters that no dual triangle joins is an edge
//    without a face, so both its ends fail;
//  * an input vertex: the same test on its incident input faces.
#include "state.cuh"

namespace acvd {

namespace {

inline unsigned mgrid(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// the corners of triangle t other than v
__device__ __forceinline__ void tri_others(const int* __restrict__ tri, int64_t t, int v, int& a, int& b) {
    const int x = tri[3 * t], y = tri[3 * t + 1], z = tri[3 * t + 2];
    if (x == v) { a = y; b = z; }
    else if (y == v) { a = z; b = x; }
    else { a = x; b = y; }
}

// how many of v's incident triangles list[p0, p1) hold corner u
template <typename L>
__device__ __forceinline__ int tri_count_corner(const int* __restrict__ tri, const L* __restrict__ list, unsigned p0,
                                                unsigned p1, int v, int u) {
    int n = 0;
    for (unsigned p = p0; p < p1; p++) {
        int a, b;
        tri_others(tri, (int64_t)list[p], v, a, b);
        n += (a == u) + (b == u);
    }
    return n;
}

// every corner on exactly two of the triangles and one cycle through all of them
template <typename L>
__device__ bool fan_is_manifold(const int* __restrict__ tri, const L* __restrict__ list, unsigned p0, unsigned p1,
                                int v) {
    const int nt = (int)(p1 - p0);
    if (nt < 2) return false;   // fewer than two edges, or edges with one face
    for (unsigned p = p0; p < p1; p++) {
        int a, b;
        tri_others(tri, (int64_t)list[p], v, a, b);
        if (a == b || a == v || b == v) return false;
        if (tri_count_corner(tri, list, p0, p1, v, a) != 2 || tri_count_corner(tri, list, p0, p1, v, b) != 2)
            return false;
    }
    int64_t prev = (int64_t)list[p0];
    int first, cur;
    tri_others(tri, prev, v, first, cur);
    int steps = 1;
    while (cur != first && steps <= nt) {
        int64_t nxt = -1;
        int nv = -1;
        for (unsigned p = p0; p < p1; p++) {
            const int64_t t = (int64_t)list[p];
            if (t == prev) continue;
            int a, b;
            tri_others(tri, t, v, a, b);
            if (a == cur) { nxt = t; nv = b; break; }
            if (b == cur) { nxt = t; nv = a; break; }
        }
        if (nxt < 0) return false;
        prev = nxt;
        cur = nv;
        steps++;
    }
    return cur == first && steps == nt;
}

__global__ void incidence_count_kernel(const int* __restrict__ dt, int64_t t, unsigned* __restrict__ cnt) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= t) return;
    atomicAdd(&cnt[dt[3 * j]], 1u);
    atomicAdd(&cnt[dt[3 * j + 1]], 1u);
    atomicAdd(&cnt[dt[3 * j + 2]], 1u);
}

__global__ void incidence_fill_kernel(const int* __restrict__ dt, int64_t t, const unsigned* __restrict__ off,
                                      unsigned* __restrict__ cursor, int* __restrict__ list) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= t) return;
    for (int q = 0; q < 3; q++) {
        const int v = dt[3 * j + q];
        list[off[v] + atomicAdd(&cursor[v], 1u)] = (int)j;
    }
}

__global__ void dual_vertex_kernel(const int* __restrict__ dt, const unsigned* __restrict__ off,
                                   const int* __restrict__ list, int k, unsigned char* __restrict__ bad) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    bad[c] = fan_is_manifold(dt, list, off[c], off[c + 1], c) ? 0 : 1;
}

// an adjacent cluster pair (across an input edge) that no dual triangle joins
__global__ void cut_edge_kernel(const int* __restrict__ edge_int, int64_t ne, const int* __restrict__ label, int k,
                                const int* __restrict__ dt, const unsigned* __restrict__ off,
                                const int* __restrict__ list, unsigned char* __restrict__ bad) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int c1 = label[edge_int[2 * e]], c2 = label[edge_int[2 * e + 1]];
    if (c1 == c2 || c1 < 0 || c2 < 0 || c1 >= k || c2 >= k) return;
    if (tri_count_corner(dt, list, off[c1], off[c1 + 1], c1, c2) == 0) {
        bad[c1] = 1;
        bad[c2] = 1;
    }
}

// items of the failing clusters: is the input vertex itself non-manifold?
__global__ void item_manifold_kernel(const int* __restrict__ label, int64_t n, int k, const int* __restrict__ orig,
                                     const uint32_t* __restrict__ vf_row, const uint32_t* __restrict__ vf_face,
                                     const int* __restrict__ tri, const int* __restrict__ row,
                                     const unsigned char* __restrict__ bad, unsigned char* __restrict__ has_nm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = label[i];
    if (c < 0 || c >= k || !bad[c]) return;
    const int v = orig[i];
    // as many faces as ring edges is implied by a single fan; check the edge count too
    const int deg = row[i + 1] - row[i];
    const unsigned f0 = vf_row[v], f1 = vf_row[v + 1];
    const bool ok = deg >= 2 && (int)(f1 - f0) == deg && fan_is_manifold(tri, vf_face, f0, f1, v);
    if (!ok) has_nm[c] = 1;
}

__global__ void issue_kernel(const unsigned char* __restrict__ bad, const unsigned char* __restrict__ has_nm,
                             const int* __restrict__ size, int k, unsigned char* __restrict__ issue) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    issue[c] = (bad[c] && size[c] > 0 && !has_nm[c]) ? 1 : 0;
}

// the output-mesh neighbours of the clusters with issues
__global__ void unfreeze_kernel(const int* __restrict__ edge_int, int64_t ne, const int* __restrict__ label, int k,
                                const unsigned char* __restrict__ issue, unsigned char* __restrict__ unf) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int c1 = label[edge_int[2 * e]], c2 = label[edge_int[2 * e + 1]];
    if (c1 == c2 || c1 < 0 || c2 < 0 || c1 >= k || c2 >= k) return;
    if (issue[c1]) unf[c2] = 1;
    if (issue[c2]) unf[c1] = 1;
}

// input edges with exactly one face (vtkSurfaceBase's Poly2 < 0 with Poly1 >= 0)
__global__ void boundary_edge_kernel(const int* __restrict__ edge_v, int64_t ne, const uint32_t* __restrict__ vf_row,
                                     const uint32_t* __restrict__ vf_face, const int* __restrict__ tri,
                                     uint32_t* __restrict__ flag) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edge_v[2 * e], b = edge_v[2 * e + 1];
    int n = 0;
    for (unsigned p = vf_row[a]; p < vf_row[a + 1]; p++) {
        const int64_t f = vf_face[p];
        n += (tri[3 * f] == b) + (tri[3 * f + 1] == b) + (tri[3 * f + 2] == b);
    }
    flag[e] = n == 1 ? 1u : 0u;
}

// the boundary edges' endpoints, their clusters, valences and coordinates
__global__ void boundary_gather_kernel(const int* __restrict__ ids, int64_t nb, const int* __restrict__ edge_v,
                                       const int* __restrict__ label_ext, const int* __restrict__ inv,
                                       const int* __restrict__ row, const double* __restrict__ xyz,
                                       BoundaryEdge* __restrict__ out) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int e = ids[b];
    const int v1 = edge_v[2 * (int64_t)e], v2 = edge_v[2 * (int64_t)e + 1];
    BoundaryEdge r;
    r.edge = e;
    r.v[0] = v1;
    r.v[1] = v2;
    r.c[0] = label_ext[v1];
    r.c[1] = label_ext[v2];
    const int i1 = inv[v1], i2 = inv[v2];
    r.deg[0] = row[i1 + 1] - row[i1];
    r.deg[1] = row[i2 + 1] - row[i2];
    for (int q = 0; q < 3; q++) {
        r.p1[q] = xyz[3 * (int64_t)v1 + q];
        r.p2[q] = xyz[3 * (int64_t)v2 + q];
    }
    out[b] = r;
}

}  // namespace

cudaError_t launch_boundary_gather(const int* ids, int64_t nb, const int* edge_v, const int* label_ext, const int* inv,
                                   const int* row, const double* xyz, BoundaryEdge* out, cudaStream_t s) {
    if (nb == 0) return cudaSuccess;
    boundary_gather_kernel<<<mgrid(nb, 256), 256, 0, s>>>(ids, nb, edge_v, label_ext, inv, row, xyz, out);
    return cudaGetLastError();
}

cudaError_t launch_dual_incidence(const int* dt, int64_t t, unsigned* cnt, const unsigned* off, unsigned* cursor,
                                  int* list, bool fill, cudaStream_t s) {
    if (t == 0) return cudaSuccess;
    if (!fill) incidence_count_kernel<<<mgrid(t, 256), 256, 0, s>>>(dt, t, cnt);
    else incidence_fill_kernel<<<mgrid(t, 256), 256, 0, s>>>(dt, t, off, cursor, list);
    return cudaGetLastError();
}

cudaError_t launch_manifold_checks(const int* dt, const unsigned* off, const int* list, int k, const int* edge_int,
                                   int64_t ne, const int* label, int64_t n, const int* orig, const uint32_t* vf_row,
                                   const uint32_t* vf_face, const int* tri, const int* row, const int* size,
                                   unsigned char* bad, unsigned char* has_nm, unsigned char* issue,
                                   unsigned char* unf, cudaStream_t s) {
    if (k > 0) dual_vertex_kernel<<<mgrid(k, 128), 128, 0, s>>>(dt, off, list, k, bad);
    if (ne > 0) cut_edge_kernel<<<mgrid(ne, 256), 256, 0, s>>>(edge_int, ne, label, k, dt, off, list, bad);
    if (n > 0)
        item_manifold_kernel<<<mgrid(n, 256), 256, 0, s>>>(label, n, k, orig, vf_row, vf_face, tri, row, bad, has_nm);
    if (k > 0) issue_kernel<<<mgrid(k, 256), 256, 0, s>>>(bad, has_nm, size, k, issue);
    if (ne > 0) unfreeze_kernel<<<mgrid(ne, 256), 256, 0, s>>>(edge_int, ne, label, k, issue, unf);
    return cudaGetLastError();
}

cudaError_t launch_boundary_edge_flags(const int* edge_v, int64_t ne, const uint32_t* vf_row, const uint32_t* vf_face,
                                       const int* tri, uint32_t* flag, cudaStream_t s) {
    if (ne == 0) return cudaSuccess;
    boundary_edge_kernel<<<mgrid(ne, 256), 256, 0, s>>>(edge_v, ne, vf_row, vf_face, tri, flag);
    return cudaGetLastError();
}

}  // namespace acvd

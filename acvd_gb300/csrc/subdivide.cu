// Midpoint subdivision of a triangle mesh, one level per launch sequence:
// vtkSurface::Subdivide (Common/vtkSurface.cxx:605-677) and the parent
// interpolation of the vertex indicator that vtkDiscreteRemeshing's
// pre-processing applies after it (DiscreteRemeshing/vtkDiscreteRemeshing.h:731-745).
//
// Output numbering is the reference's: the old vertices keep their ids, edge e
// gives vertex nV + e at its midpoint, face f gives faces 4f .. 4f+3 as
// (V1,V4,V6), (V4,V2,V5), (V5,V3,V6), (V4,V5,V6) with V4, V5, V6 the children
// of edges V1V2, V2V3, V3V1.  The reference stores the new mesh's points in a
// float vtkPoints, so every output coordinate is the float nearest to the FP64
// value (the old point, or 0.5 (P1 + P2)).
#include "state.cuh"

namespace acvd {

namespace {

inline unsigned sgrid(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

__global__ void subdiv_slot_edges_kernel(const int* __restrict__ edge_v, int64_t ne, int64_t nv,
                                         const int* __restrict__ row, const int* __restrict__ col,
                                         int* __restrict__ slot_edge) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edge_v[2 * e], b = edge_v[2 * e + 1];
    if (a < 0 || b < 0 || a >= nv || b >= nv) return;   // left -1: the faces on it are reported
    for (int p = row[a]; p < row[a + 1]; p++)
        if (col[p] == b) { slot_edge[p] = (int)e; break; }
    for (int p = row[b]; p < row[b + 1]; p++)
        if (col[p] == a) { slot_edge[p] = (int)e; break; }
}

// float-rounded copy of the old points, then one midpoint per edge
__global__ void subdiv_points_kernel(const double* __restrict__ xyz, int64_t nv, const int* __restrict__ edge_v,
                                     int64_t ne, const double* __restrict__ ind, double* __restrict__ out_xyz,
                                     int* __restrict__ parent1, int* __restrict__ parent2,
                                     double* __restrict__ out_ind) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv + ne) return;
    if (i < nv) {
        for (int c = 0; c < 3; c++) out_xyz[3 * i + c] = (double)__double2float_rn(xyz[3 * i + c]);
        if (out_ind) out_ind[i] = ind[i];
        return;
    }
    const int64_t e = i - nv;
    const int a = edge_v[2 * e], b = edge_v[2 * e + 1];
    if (a < 0 || b < 0 || a >= nv || b >= nv) return;
    for (int c = 0; c < 3; c++) {
        const double m = 0.5 * (xyz[3 * (int64_t)a + c] + xyz[3 * (int64_t)b + c]);
        out_xyz[3 * i + c] = (double)__double2float_rn(m);
    }
    parent1[e] = a;
    parent2[e] = b;
    // CellsIndicators2[i] = (CellsIndicators2[Parent1[i]] + CellsIndicators2[Parent2[i]]) * 0.5
    if (out_ind) out_ind[i] = (ind[a] + ind[b]) * 0.5;
}

__device__ __forceinline__ int subdiv_edge_of(const int* __restrict__ row, const int* __restrict__ col,
                                              const int* __restrict__ slot_edge, int a, int b) {
    for (int p = row[a]; p < row[a + 1]; p++)
        if (col[p] == b) return slot_edge[p];
    return -1;
}

__global__ void subdiv_faces_kernel(const int* __restrict__ tri, int64_t nf, int64_t nv, const int* __restrict__ row,
                                    const int* __restrict__ col, const int* __restrict__ slot_edge,
                                    int* __restrict__ out_tri, unsigned int* __restrict__ missing) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int v1 = tri[3 * f], v2 = tri[3 * f + 1], v3 = tri[3 * f + 2];
    if (v1 == v2 || v1 < 0 || v2 < 0 || v3 < 0 || v1 >= nv || v2 >= nv || v3 >= nv) {
        // an inactive face for vtkSurface, or a vertex id out of range: reported, not subdivided
        atomicAdd(missing, 1u);
        return;
    }
    const int e12 = subdiv_edge_of(row, col, slot_edge, v1, v2);
    const int e23 = subdiv_edge_of(row, col, slot_edge, v2, v3);
    const int e31 = subdiv_edge_of(row, col, slot_edge, v3, v1);
    if ((e12 | e23 | e31) < 0) {
        atomicAdd(missing, 1u);
        return;
    }
    const int v4 = (int)(nv + e12), v5 = (int)(nv + e23), v6 = (int)(nv + e31);
    int* o = out_tri + 12 * f;
    o[0] = v1; o[1] = v4;  o[2] = v6;
    o[3] = v4; o[4] = v2;  o[5] = v5;
    o[6] = v5; o[7] = v3;  o[8] = v6;
    o[9] = v4; o[10] = v5; o[11] = v6;
}

}  // namespace

cudaError_t launch_subdivide(const double* xyz, int64_t nv, const int* tri, int64_t nf, const int* row,
                             const int* col, const int* edge_v, int64_t ne, const double* ind, int* slot_edge,
                             double* out_xyz, int* out_tri, int* parent1, int* parent2, double* out_ind,
                             unsigned int* missing, cudaStream_t s) {
    cudaError_t err = cudaMemsetAsync(slot_edge, 0xff, 2 * (size_t)ne * sizeof(int), s);
    if (err != cudaSuccess) return err;
    if (ne > 0) subdiv_slot_edges_kernel<<<sgrid(ne, 256), 256, 0, s>>>(edge_v, ne, nv, row, col, slot_edge);
    if (nv + ne > 0)
        subdiv_points_kernel<<<sgrid(nv + ne, 256), 256, 0, s>>>(xyz, nv, edge_v, ne, ind, out_xyz, parent1, parent2,
                                                                  out_ind);
    if (nf > 0) subdiv_faces_kernel<<<sgrid(nf, 256), 256, 0, s>>>(tri, nf, nv, row, col, slot_edge, out_tri, missing);
    return cudaGetLastError();
}

}  // namespace acvd

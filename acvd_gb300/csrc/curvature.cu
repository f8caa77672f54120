// Per-vertex curvature for vertex clustering: the curvature indicator and the
// principal directions that vtkDiscreteRemeshing's pre-processing computes with
// vtkCurvatureMeasure (DiscreteRemeshing/vtkDiscreteRemeshing.h:630-637):
// polynomial fitting (method 1) on the faces of the vertex 3-ring.
//
// One thread per vertex, FP64.  This file is compiled without FMA contraction
// (build.py) and every expression keeps the operation order of the CPU
// restatement, so that each value equals it bit for bit (the divisions and
// square roots are the correctly rounded IEEE operations on both sides).
#include "../../include/acvd_gpu.h"
#include "primitives.cuh"
#include "state.cuh"

namespace acvd {

constexpr int kCurvMaxF = 192;    // faces of one 3-ring
constexpr int kCurvMaxV = 384;    // vertices queued for one ring step
constexpr int kCurvMaxVis = 96;   // vertices of rings 0..2

// Faces of edge e: the first two faces, in increasing id, holding both of its
// endpoints (the reference attaches faces to an edge in face order,
// Common/vtkSurfaceBase.cxx:1166-1221).  Original vertex ids.
__global__ void edge_faces_kernel(const int* __restrict__ edge_v, int64_t ne, const int* __restrict__ tri,
                                  const uint32_t* __restrict__ vf_row, const uint32_t* __restrict__ vf_face,
                                  int2* __restrict__ poly) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edge_v[2 * e], b = edge_v[2 * e + 1];
    int f1 = -1, f2 = -1;
    for (uint32_t t = vf_row[a]; t < vf_row[a + 1] && f2 < 0; t++) {
        const int f = (int)vf_face[t];
        if (tri[3 * f] == b || tri[3 * f + 1] == b || tri[3 * f + 2] == b) {
            if (f1 < 0) f1 = f;
            else f2 = f;
        }
    }
    poly[e] = make_int2(f1, f2);
}

// Edge id of every ring slot of the internal CSR (edges in internal ids).
__global__ void slot_edges_kernel(const int* __restrict__ edge_int, int64_t ne, const int* __restrict__ row,
                                  const int* __restrict__ col, int* __restrict__ slot_edge) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edge_int[2 * e], b = edge_int[2 * e + 1];
    for (int p = row[a]; p < row[a + 1]; p++)
        if (col[p] == b) { slot_edge[p] = (int)e; break; }
    for (int p = row[b]; p < row[b + 1]; p++)
        if (col[p] == a) { slot_edge[p] = (int)e; break; }
}

// Per face, once: unit normal, area and area-weighted barycentre, the values the
// fit reads for every vertex whose 3-ring holds the face.
struct FaceProps {
    double n[3];
    double area;
    double bary[3];
    double pad;
};

struct CurvMesh {
    const double* xyz;
    const int* tri;
    const FaceProps* fp;
    int64_t nv;
    const int* row;        // internal ring CSR
    const int* col;
    const int* perm;       // item -> original vertex
    const int* inv;        // original vertex -> item
    const int* slot_edge;
    const int2* poly;
};

// area by the side-length form (Common/vtkSurface.cxx:1283) and the
// area-weighted vertex mean (vtkSurface::GetCellMassProperties, :1380-1419)
__device__ void curv_face_mass(const double p1[3], const double p2[3], const double p3[3], double& area,
                               double bary[3]) {
    const double d12[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
    const double d23[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
    const double d31[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    const double a = d12[0] * d12[0] + d12[1] * d12[1] + d12[2] * d12[2];
    const double b = d23[0] * d23[0] + d23[1] * d23[1] + d23[2] * d23[2];
    const double c = d31[0] * d31[0] + d31[1] * d31[1] + d31[2] * d31[2];
    const double a2 = 0.25 * sqrt(fabs(4.0 * a * c - (a - b + c) * (a - b + c)));
    for (int i = 0; i < 3; i++) bary[i] = 0.0 + a2 * (p1[i] + p2[i] + p3[i]) / 3.0;
    area = 0.0 + a2;
    if (area > 0)
        for (int i = 0; i < 3; i++) bary[i] /= area;
}

// unit normal from (x3 - x2) x (x1 - x2)
__device__ void curv_normal(const double x1[3], const double x2[3], const double x3[3], double n[3]) {
    const double a[3] = {x3[0] - x2[0], x3[1] - x2[1], x3[2] - x2[2]};
    const double b[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
    n[0] = a[1] * b[2] - a[2] * b[1];
    n[1] = a[2] * b[0] - a[0] * b[2];
    n[2] = a[0] * b[1] - a[1] * b[0];
    const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (l != 0.0) { n[0] /= l; n[1] /= l; n[2] /= l; }
}

__device__ __forceinline__ void curv_normalize(double a[3]) {
    const double n = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (n != 0.0) { a[0] /= n; a[1] /= n; a[2] /= n; }
}

__device__ __forceinline__ void curv_cross(const double a[3], const double b[3], double c[3]) {
    const double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    c[0] = x; c[1] = y; c[2] = z;
}

__device__ __forceinline__ double curv_dot(const double a[3], const double b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__global__ void face_props_kernel(const double* __restrict__ xyz, const int* __restrict__ tri, int64_t nf,
                                  FaceProps* __restrict__ fp) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double p1[3], p2[3], p3[3];
    for (int k = 0; k < 3; k++) {
        p1[k] = xyz[3 * (int64_t)tri[3 * f] + k];
        p2[k] = xyz[3 * (int64_t)tri[3 * f + 1] + k];
        p3[k] = xyz[3 * (int64_t)tri[3 * f + 2] + k];
    }
    FaceProps r;
    curv_normal(p1, p2, p3, r.n);
    curv_face_mass(p1, p2, p3, r.area, r.bary);
    r.pad = 0.0;
    fp[f] = r;
}

// Inverse of the n x n matrix a by LU decomposition with partial pivoting
// (Doolittle), one substitution per unit vector; 0 when a pivot is exactly zero.
template <int N>
__device__ int curv_lu_invert(const double a[N][N], double ai[N][N]) {
    double lu[N][N];
    int piv[N];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) lu[i][j] = a[i][j];
    for (int k = 0; k < N; k++) {
        int p = k;
        double best = fabs(lu[k][k]);
        for (int i = k + 1; i < N; i++) {
            const double v = fabs(lu[i][k]);
            if (v > best) { best = v; p = i; }
        }
        if (best == 0.0) return 0;
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < N; j++) { const double t = lu[k][j]; lu[k][j] = lu[p][j]; lu[p][j] = t; }
        const double d = lu[k][k];
        for (int i = k + 1; i < N; i++) {
            const double f = lu[i][k] / d;
            lu[i][k] = f;
            for (int j = k + 1; j < N; j++) lu[i][j] -= f * lu[k][j];
        }
    }
    for (int c = 0; c < N; c++) {
        double x[N];
        for (int i = 0; i < N; i++) x[i] = (i == c) ? 1.0 : 0.0;
        for (int k = 0; k < N; k++)
            if (piv[k] != k) { const double t = x[k]; x[k] = x[piv[k]]; x[piv[k]] = t; }
        for (int i = 0; i < N; i++)
            for (int j = 0; j < i; j++) x[i] -= lu[i][j] * x[j];
        for (int i = N - 1; i >= 0; i--) {
            for (int j = i + 1; j < N; j++) x[i] -= lu[i][j] * x[j];
            x[i] /= lu[i][i];
        }
        for (int i = 0; i < N; i++) ai[i][c] = x[i];
    }
    return 1;
}

// Eigen-decomposition of the symmetric 2x2 matrix given by the upper triangle of
// a (cyclic Jacobi; Golub & Van Loan sec. 8.5): w decreasing, unit eigenvectors in
// the columns of v.
__device__ void curv_jacobi2(const double a[2][2], double w[2], double v[2][2]) {
    double m[2][2] = {{a[0][0], a[0][1]}, {a[0][1], a[1][1]}};
    v[0][0] = 1.0; v[0][1] = 0.0; v[1][0] = 0.0; v[1][1] = 1.0;
    for (int sweep = 0; sweep < 64; sweep++) {
        const double off = m[0][1] * m[0][1];
        if (off == 0.0) break;
        const double apq = m[0][1];
        if (apq == 0.0) continue;
        const double theta = (m[1][1] - m[0][0]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 2; k++) {
            const double mkp = m[k][0], mkq = m[k][1];
            m[k][0] = c * mkp - s * mkq;
            m[k][1] = s * mkp + c * mkq;
        }
        for (int k = 0; k < 2; k++) {
            const double mpk = m[0][k], mqk = m[1][k];
            m[0][k] = c * mpk - s * mqk;
            m[1][k] = s * mpk + c * mqk;
        }
        m[0][1] = m[1][0] = 0.0;
        for (int k = 0; k < 2; k++) {
            const double vkp = v[k][0], vkq = v[k][1];
            v[k][0] = c * vkp - s * vkq;
            v[k][1] = s * vkp + c * vkq;
        }
    }
    w[0] = m[0][0];
    w[1] = m[1][1];
    if (w[1] > w[0]) {
        const double t = w[0]; w[0] = w[1]; w[1] = t;
        for (int k = 0; k < 2; k++) { const double u = v[k][0]; v[k][0] = v[k][1]; v[k][1] = u; }
    }
}

// vtkSinglePolynomialMeasure::ComputeFitting (Common/vtkCurvatureMeasure.cxx:188-505)
// on the faces fl[0..nf): returns sqrt(k1^2 + k2^2), info = principal directions
// scaled by sqrt|k|, the larger |k| first.
__device__ double curv_fit(const CurvMesh& m, const int* fl, int nf, double* xs, double* ys, double* zs,
                           double info[6]) {
    double sarea = 0, origin[3] = {0, 0, 0}, frame[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int j = 0; j < nf; j++) {
        const FaceProps& q = m.fp[fl[j]];
        const double area = q.area;
        for (int k = 0; k < 3; k++) {
            origin[k] += area * q.bary[k];
            frame[0][k] += area * q.n[k];
        }
        sarea += area;
    }
    for (int j = 0; j < 3; j++) origin[j] = origin[j] / sarea;
    curv_normalize(frame[0]);
    for (int k = 0; k < 3; k++) frame[2][k] = frame[0][k];
    frame[1][1] = frame[2][0]; frame[1][2] = frame[2][1]; frame[1][0] = frame[2][2];
    curv_cross(frame[1], frame[2], frame[0]);
    curv_normalize(frame[0]);
    curv_cross(frame[2], frame[0], frame[1]);
    for (int i = 0; i < 6; i++) info[i] = 0;
    if (nf <= 6) return 0;
    double h = 0;
    for (int j = 0; j < nf; j++) {
        const FaceProps& fq = m.fp[fl[j]];
        double bary[3] = {fq.bary[0], fq.bary[1], fq.bary[2]};
        for (int k = 0; k < 3; k++) bary[k] -= origin[k];
        const double x = curv_dot(bary, frame[0]), y = curv_dot(bary, frame[1]), z = curv_dot(bary, frame[2]);
        xs[j] = x; ys[j] = y; zs[j] = z;
        h += sqrt(x * x + y * y);
    }
    h = h / ((double)nf);
    // normal equations of the conditioned Vandermonde rows (upper half, mirrored)
    double xxt[6][6], xxti[6][6], xyt[6], q[6];
    for (int i = 0; i < 6; i++) {
        xyt[i] = 0.0;
        for (int j = 0; j < 6; j++) xxt[i][j] = 0.0;
    }
    for (int k = 0; k < nf; k++) {
        const double x = xs[k], y = ys[k];
        double r[6] = {1.0, x, y, x * x, x * y, y * y};
        r[1] /= h; r[2] /= h; r[3] /= h * h; r[4] /= h * h; r[5] /= h * h;
        for (int i = 0; i < 6; i++) {
            for (int j = i; j < 6; j++) xxt[i][j] += r[i] * r[j];
            xyt[i] += r[i] * zs[k];
        }
    }
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < i; j++) xxt[i][j] = xxt[j][i];
    if (!curv_lu_invert<6>(xxt, xxti)) return 0;
    for (int i = 0; i < 6; i++) {
        q[i] = 0.0;
        for (int k = 0; k < 6; k++) q[i] += xxti[i][k] * xyt[k];
    }
    q[1] /= h; q[2] /= h; q[3] /= h * h; q[4] /= h * h; q[5] /= h * h;
    const double E = 1.0 + q[1] * q[1], F = q[1] * q[2], G = 1.0 + q[2] * q[2];
    const double e = 2.0 * q[3] / sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    const double ff = 2.0 * q[4] / sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    const double g = 2.0 * q[5] / sqrt(q[1] * q[1] + 1.0 + q[2] * q[2]);
    double A[2][2] = {{E, F}, {F, G}}, B[2][2];
    if (!curv_lu_invert<2>(A, B)) return 0;
    A[0][0] = -(e * B[0][0] + ff * B[1][0]);
    A[1][0] = -(e * B[0][1] + ff * B[1][1]);
    A[0][1] = -(ff * B[0][0] + g * B[1][0]);
    A[1][1] = -(ff * B[0][1] + g * B[1][1]);
    double ev[2], evec[2][2];
    curv_jacobi2(A, ev, evec);
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 3; k++) info[k + 3 * j] += sqrt(fabs(ev[j])) * evec[i][j] * frame[i][k];
    if (fabs(ev[0]) < fabs(ev[1]))
        for (int i = 0; i < 3; i++) { const double t = info[i]; info[i] = info[i + 3]; info[i + 3] = t; }
    return sqrt(ev[0] * ev[0] + ev[1] * ev[1]);
}

// One vertex (original id v): the faces of its 3-ring in the reference's order
// (vtkNeighbourhoodComputation::ComputeNRingCells, Common/vtkNeighbourhoodComputation.cxx:38-100:
// the vertex's own faces, then ring by ring the faces of the edges of each vertex
// not yet visited), then the fit.  A neighbourhood larger than the buffers counts
// in *overflow and leaves the vertex's outputs at zero.
__global__ void __launch_bounds__(64) curvature_kernel(CurvMesh m, double* __restrict__ indicator,
                                                       float* __restrict__ dirs,
                                                       unsigned long long* __restrict__ overflow) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nv) return;
    int fl[kCurvMaxF];
    int vis[kCurvMaxVis];
    int lists[2][kCurvMaxV];
    int nf = 0, nvis = 0;
    bool ok = true;
    auto add_face = [&](int f) {
        for (int i = 0; i < nf; i++)
            if (fl[i] == f) return;
        if (nf < kCurvMaxF) fl[nf++] = f;
        else ok = false;
    };
    {
        const int t = m.inv[v];
        for (int p = m.row[t]; p < m.row[t + 1]; p++) {
            const int e = m.slot_edge[p];
            if (e < 0) continue;
            const int2 pf = m.poly[e];
            if (pf.x >= 0) add_face(pf.x);
            if (pf.y >= 0) add_face(pf.y);
        }
    }
    int cur = 0, ncur = 1;
    lists[0][0] = (int)v;
    for (int r = 0; r < 3 && ok; r++) {
        int nnext = 0;
        for (int k = 0; k < ncur && ok; k++) {
            const int u = lists[cur][k];
            bool seen = false;
            for (int i = 0; i < nvis; i++) seen |= vis[i] == u;
            if (seen) continue;
            if (nvis == kCurvMaxVis) { ok = false; break; }
            vis[nvis++] = u;
            const int tu = m.inv[u];
            for (int p = m.row[tu]; p < m.row[tu + 1]; p++) {
                if (nnext == kCurvMaxV) { ok = false; break; }
                lists[cur ^ 1][nnext++] = m.perm[m.col[p]];
                const int e = m.slot_edge[p];
                if (e < 0) continue;
                const int2 pf = m.poly[e];
                if (pf.x >= 0) {
                    add_face(pf.x);
                    if (pf.y >= 0) add_face(pf.y);
                }
            }
        }
        cur ^= 1;
        ncur = nnext;
    }
    double info[6] = {0, 0, 0, 0, 0, 0};
    double ind = 0.0;
    if (ok) {
        double xs[kCurvMaxF], ys[kCurvMaxF], zs[kCurvMaxF];
        ind = curv_fit(m, fl, nf, xs, ys, zs, info);
    } else {
        atomicAdd(overflow, 1ull);
    }
    indicator[v] = ind;
    for (int i = 0; i < 6; i++) dirs[6 * v + i] = (float)info[i];
}

static inline unsigned cgrid(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

size_t curvature_face_bytes(int64_t nf) { return (size_t)nf * sizeof(FaceProps); }

cudaError_t launch_curvature(const double* xyz, const int* tri, int64_t nv, int64_t nf, int64_t ne,
                             const int* edge_v, const int* edge_int, const uint32_t* vf_row, const uint32_t* vf_face,
                             const int* row, const int* col, const int* perm, const int* inv, int2* poly,
                             int* slot_edge, void* face_work, double* indicator, float* dirs,
                             unsigned long long* overflow, cudaStream_t s) {
    if (nv == 0) return cudaSuccess;
    cudaError_t err = cudaMemsetAsync(slot_edge, 0xff, 2 * ne * sizeof(int), s);   // -1: no edge
    if (err != cudaSuccess) return err;
    g_launches += 4;
    FaceProps* fp = (FaceProps*)face_work;
    face_props_kernel<<<cgrid(nf, 256), 256, 0, s>>>(xyz, tri, nf, fp);
    edge_faces_kernel<<<cgrid(ne, 256), 256, 0, s>>>(edge_v, ne, tri, vf_row, vf_face, poly);
    slot_edges_kernel<<<cgrid(ne, 256), 256, 0, s>>>(edge_int, ne, row, col, slot_edge);
    CurvMesh m{xyz, tri, fp, nv, row, col, perm, inv, slot_edge, poly};
    curvature_kernel<<<cgrid(nv, 64), 64, 0, s>>>(m, indicator, dirs, overflow);
    return cudaGetLastError();
}

}  // namespace acvd

// Adjoint of the clustering energy for a fixed clustering (FP64 throughout).
//
// Forward, as a function of the vertex positions x and the per-vertex densities
// rho (the curvature-indicator slot of the metric, weight = area * rho^g):
//   face f:    cr = (p1 - p0) x (p2 - p0), area = |cr| / 2, unit normal n = cr / |cr|
//              (Common/vtkSurface.cxx:1283 area, Common/vtkQuadricTools.cxx:56-79 plane quadric)
//   vertex i:  a_i = sum_f area_f / 3, w_i = a_i rho_i^g (clamped weights are constants),
//              A_i = sum_f n n^T, b_i = A_i x_i (x_i lies on every adjacent plane)
//   cluster k: S = sum w x, W = sum w, A = sum A_i, b = sum b_i, m = S / W,
//              c = m + P (b - A m) with P the thresholded pseudo-inverse of A whose kept
//              eigenvalues are those of the forward pass (rank held fixed;
//              vtkQuadricTools.cxx:83-163), E_k = W |c|^2 - 2 c.S (vtkQEMetricForClustering.h:194-208)
// Backward: the vector-Jacobian product of L = gE * sum_k E_k + sum_k gC_k . c_k
// with respect to x and rho.  Cluster sums are recomputed, not stored.
#include <cmath>

#include "primitives.cuh"
#include "state.cuh"

namespace acvd {


constexpr int kClStride = 32;   // doubles per cluster record

__global__ void adj_face_fwd(AdjState a) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.nf) return;
    const int i0 = a.tri[3 * f], i1 = a.tri[3 * f + 1], i2 = a.tri[3 * f + 2];
    double e1[3], e2[3];
    for (int d = 0; d < 3; d++) {
        e1[d] = a.x[3 * i1 + d] - a.x[3 * i0 + d];
        e2[d] = a.x[3 * i2 + d] - a.x[3 * i0 + d];
    }
    const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double L = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    a.flen[f] = L;
    a.farea[f] = 0.5 * L;
    for (int d = 0; d < 3; d++) a.fn[3 * f + d] = L > 0.0 ? cr[d] / L : 0.0;
}

__global__ void adj_vertex_fwd(AdjState a) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= a.nv) return;
    double area = 0.0, A[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t j = a.vf_row[v]; j < a.vf_row[v + 1]; j++) {
        const uint32_t f = a.vf_face[j];
        area += a.farea[f] / 3.0;
        const double n0 = a.fn[3 * f], n1 = a.fn[3 * f + 1], n2 = a.fn[3 * f + 2];
        A[0] += n0 * n0; A[1] += n0 * n1; A[2] += n0 * n2; A[3] += n1 * n1; A[4] += n1 * n2; A[5] += n2 * n2;
    }
    a.va[v] = area;
    for (int j = 0; j < 6; j++) a.vA[6 * v + j] = A[j];
    a.vw[v] = a.rho ? area * pow(a.rho[v], a.grad) : area;
}

__global__ void adj_clamp(AdjState a, const double* wsum, double ratio) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= a.nv) return;
    const double mean = *wsum / (double)a.nv;
    double w = a.vw[v];
    unsigned char c = 0;
    if (w > mean * ratio) { w = mean * ratio; c = 1; }
    if (w < mean / ratio) { w = mean / ratio; c = 1; }
    a.vw[v] = w;
    a.vclamp[v] = c;
}

// one warp per cluster over its items (sorted by cluster): FP64 sums, fixed order
__global__ void adj_cluster_sums(AdjState a, const uint32_t* __restrict__ sorted, const uint32_t* __restrict__ off,
                                 const uint32_t* __restrict__ cnt) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= a.k) return;
    double s[13];
    for (int q = 0; q < 13; q++) s[q] = 0.0;
    for (uint32_t j = lane; j < cnt[w]; j += 32) {
        const uint32_t i = sorted[off[w] + j];
        const double wi = a.vw[i];
        const double xi[3] = {a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2]};
        const double* Ai = a.vA + 6 * (int64_t)i;
        s[0] += wi * xi[0]; s[1] += wi * xi[1]; s[2] += wi * xi[2]; s[3] += wi;
        for (int q = 0; q < 6; q++) s[4 + q] += Ai[q];
        s[10] += Ai[0] * xi[0] + Ai[1] * xi[1] + Ai[2] * xi[2];
        s[11] += Ai[1] * xi[0] + Ai[3] * xi[1] + Ai[4] * xi[2];
        s[12] += Ai[2] * xi[0] + Ai[4] * xi[1] + Ai[5] * xi[2];
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int q = 0; q < 13; q++) s[q] += __shfl_xor_sync(kFull, s[q], o);
    if (lane == 0)
        for (int q = 0; q < 13; q++) a.cl[w * kClStride + q] = s[q];
}

ACVD_DEV void smul(const double a[6], const double v[3], double o[3]) {
    o[0] = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
    o[1] = a[1] * v[0] + a[3] * v[1] + a[4] * v[2];
    o[2] = a[2] * v[0] + a[4] * v[1] + a[5] * v[2];
}

// per cluster: placement, energy, and the cotangents of S, W, A, b
// gE: the cotangent of the total energy, read from dgE (device) when that is given
__global__ void adj_cluster(AdjState a, int metric, int level, double thr, double gE_host, const double* dgE,
                            const double* __restrict__ gC, double* __restrict__ cent) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.k) return;
    const double gE = dgE ? *dgE : gE_host;
    double* r0 = a.cl + k * kClStride;
    const double S[3] = {r0[0], r0[1], r0[2]};
    const double W = r0[3];
    for (int q = 13; q < kClStride; q++) r0[q] = 0.0;
    a.ek[k] = 0.0;
    if (!(W > 0.0)) return;
    const double A[6] = {r0[4], r0[5], r0[6], r0[7], r0[8], r0[9]};
    const double b[3] = {r0[10], r0[11], r0[12]};
    const double m[3] = {S[0] / W, S[1] / W, S[2] / W};
    double Am[3];
    smul(A, m, Am);
    const double r[3] = {b[0] - Am[0], b[1] - Am[1], b[2] - Am[2]};
    // eigen-decomposition and the kept set (the forward's rank decision)
    double lam[3], V[3][3];
    jacobi_eig3<double>(A, lam, V, 64);
    double aw[3] = {fabs(lam[0]), fabs(lam[1]), fabs(lam[2])};
    const double mx = fmax(aw[0], fmax(aw[1], aw[2]));
    bool keep[3] = {false, false, false};
    if (metric != kIso) {
        int used = 0;
        for (int it = 0; it < 3; it++) {
            int im = 0;
            if (aw[1] > aw[im]) im = 1;
            if (aw[2] > aw[im]) im = 2;
            if (mx > 0.0 && aw[im] > thr * mx && used < level) { keep[im] = true; used++; }
            aw[im] = -1.0;
        }
    }
    // P = sum_kept v v^T / lambda
    double P[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 3; j++) {
        if (!keep[j]) continue;
        const double il = 1.0 / lam[j];
        P[0] += V[0][j] * V[0][j] * il; P[1] += V[0][j] * V[1][j] * il; P[2] += V[0][j] * V[2][j] * il;
        P[3] += V[1][j] * V[1][j] * il; P[4] += V[1][j] * V[2][j] * il; P[5] += V[2][j] * V[2][j] * il;
    }
    double Pr[3];
    smul(P, r, Pr);
    const double c[3] = {m[0] + Pr[0], m[1] + Pr[1], m[2] + Pr[2]};
    const double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    const double E = cc * W - 2.0 * (c[0] * S[0] + c[1] * S[1] + c[2] * S[2]);
    r0[13] = E;
    a.ek[k] = E;
    r0[14] = c[0]; r0[15] = c[1]; r0[16] = c[2];
    if (cent) { cent[3 * k] = c[0]; cent[3 * k + 1] = c[1]; cent[3 * k + 2] = c[2]; }
    // cotangent of c
    double u[3];
    for (int d = 0; d < 3; d++) u[d] = gE * 2.0 * W * (c[d] - m[d]) + (gC ? gC[3 * k + d] : 0.0);
    // M^T u = u - A P u   (M = I - P A, both symmetric)
    double Pu[3], APu[3];
    smul(P, u, Pu);
    smul(A, Pu, APu);
    const double Mu[3] = {u[0] - APu[0], u[1] - APu[1], u[2] - APu[2]};
    double GS[3];
    for (int d = 0; d < 3; d++) GS[d] = -2.0 * gE * c[d] + Mu[d] / W;
    const double GW = gE * cc - (Mu[0] * m[0] + Mu[1] * m[1] + Mu[2] * m[2]) / W;
    // b enters through P b: G_b = P u ; A enters through -P A m and through P itself
    double GA[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) GA[i][j] = -0.5 * (Pu[i] * m[j] + Pu[j] * m[i]);
    // d(u^T P r) with P = sum_kept v_j v_j^T / lam_j (first-order eigen perturbation)
    double uv[3], rv[3];
    for (int j = 0; j < 3; j++) {
        uv[j] = u[0] * V[0][j] + u[1] * V[1][j] + u[2] * V[2][j];
        rv[j] = r[0] * V[0][j] + r[1] * V[1][j] + r[2] * V[2][j];
    }
    for (int j = 0; j < 3; j++) {
        if (!keep[j]) continue;
        // eigenvalue term: -(u.v)(v.r)/lam^2 * v v^T
        const double t = -uv[j] * rv[j] / (lam[j] * lam[j]);
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) GA[p][q] += t * V[p][j] * V[q][j];
        for (int l = 0; l < 3; l++) {
            if (l == j) continue;
            double coef;
            if (keep[l]) {
                if (l < j) continue;   // kept pair handled once: 1/(lj(lj-ll)) + 1/(ll(ll-lj)) = -1/(lj ll)
                coef = -1.0 / (lam[j] * lam[l]);
            } else {
                coef = 1.0 / (lam[j] * (lam[j] - lam[l]));
            }
            const double s = coef * (uv[l] * rv[j] + uv[j] * rv[l]);
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) GA[p][q] += 0.5 * s * (V[p][l] * V[q][j] + V[p][j] * V[q][l]);
        }
    }
    r0[17] = GS[0]; r0[18] = GS[1]; r0[19] = GS[2];
    r0[20] = GW;
    // compact symmetric: off-diagonal entries appear twice in A = sum n n^T
    r0[21] = GA[0][0]; r0[22] = GA[0][1] + GA[1][0]; r0[23] = GA[0][2] + GA[2][0];
    r0[24] = GA[1][1]; r0[25] = GA[1][2] + GA[2][1]; r0[26] = GA[2][2];
    r0[27] = Pu[0]; r0[28] = Pu[1]; r0[29] = Pu[2];
}

// weight cotangent of vertex v: dL/dw = G_S . x + G_W
ACVD_DEV double vertex_gw(const AdjState& a, int64_t v, const double* g) {
    return g[17] * a.x[3 * v] + g[18] * a.x[3 * v + 1] + g[19] * a.x[3 * v + 2] + g[20];
}

// per face: cotangents of its area and unit normal from its three corners'
// items, then of its corner positions
__global__ void adj_face_bwd(AdjState a) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.nf) return;
    const double n[3] = {a.fn[3 * f], a.fn[3 * f + 1], a.fn[3 * f + 2]};
    double g_area = 0.0, g_n[3] = {0, 0, 0};
    for (int j = 0; j < 3; j++) {
        const int v = a.tri[3 * f + j];
        const int k = a.label[v];
        if (k < 0 || k >= a.k) continue;
        const double* g = a.cl + (int64_t)k * kClStride;
        if (!a.vclamp[v]) {
            const double rg = a.rho ? pow(a.rho[v], a.grad) : 1.0;
            g_area += vertex_gw(a, v, g) * rg / 3.0;
        }
        // A_v gets n n^T, b_v gets n n^T x_v
        const double GA[6] = {g[21], g[22], g[23], g[24], g[25], g[26]};
        const double Gb[3] = {g[27], g[28], g[29]};
        const double xv[3] = {a.x[3 * v], a.x[3 * v + 1], a.x[3 * v + 2]};
        // d(sum_pq GA_pq n_p n_q) / dn with the compact weights (off-diagonals counted once)
        const double Gn[3] = {2.0 * GA[0] * n[0] + GA[1] * n[1] + GA[2] * n[2],
                              GA[1] * n[0] + 2.0 * GA[3] * n[1] + GA[4] * n[2],
                              GA[2] * n[0] + GA[4] * n[1] + 2.0 * GA[5] * n[2]};
        const double nx = n[0] * xv[0] + n[1] * xv[1] + n[2] * xv[2];
        const double gbn = Gb[0] * n[0] + Gb[1] * n[1] + Gb[2] * n[2];
        for (int d = 0; d < 3; d++) g_n[d] += Gn[d] + nx * Gb[d] + gbn * xv[d];
    }
    const double L = a.flen[f];
    double g_cr[3] = {0, 0, 0};
    if (L > 0.0) {
        const double ngn = n[0] * g_n[0] + n[1] * g_n[1] + n[2] * g_n[2];
        for (int d = 0; d < 3; d++) g_cr[d] = 0.5 * g_area * n[d] + (g_n[d] - n[d] * ngn) / L;
    }
    const int i0 = a.tri[3 * f], i1 = a.tri[3 * f + 1], i2 = a.tri[3 * f + 2];
    double e1[3], e2[3];
    for (int d = 0; d < 3; d++) {
        e1[d] = a.x[3 * i1 + d] - a.x[3 * i0 + d];
        e2[d] = a.x[3 * i2 + d] - a.x[3 * i0 + d];
    }
    // cr = e1 x e2: g_e1 = e2 x g_cr, g_e2 = g_cr x e1
    const double ge1[3] = {e2[1] * g_cr[2] - e2[2] * g_cr[1], e2[2] * g_cr[0] - e2[0] * g_cr[2],
                           e2[0] * g_cr[1] - e2[1] * g_cr[0]};
    const double ge2[3] = {g_cr[1] * e1[2] - g_cr[2] * e1[1], g_cr[2] * e1[0] - g_cr[0] * e1[2],
                           g_cr[0] * e1[1] - g_cr[1] * e1[0]};
    double* out = a.corner + 9 * f;
    for (int d = 0; d < 3; d++) {
        out[d] = -ge1[d] - ge2[d];
        out[3 + d] = ge1[d];
        out[6 + d] = ge2[d];
    }
}

__global__ void adj_vertex_bwd(AdjState a, double* __restrict__ gx, double* __restrict__ grho) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= a.nv) return;
    double g[3] = {0, 0, 0};
    const int k = a.label[v];
    double gw = 0.0;
    if (k >= 0 && k < a.k) {
        const double* c = a.cl + (int64_t)k * kClStride;
        gw = vertex_gw(a, v, c);
        const double w = a.vw[v];
        const double* Av = a.vA + 6 * v;
        const double Gb[3] = {c[27], c[28], c[29]};
        double AGb[3];
        smul(Av, Gb, AGb);
        for (int d = 0; d < 3; d++) g[d] += w * c[17 + d] + AGb[d];
    }
    for (uint32_t j = a.vf_row[v]; j < a.vf_row[v + 1]; j++) {
        const uint32_t f = a.vf_face[j];
        int corner = 0;
        if (a.tri[3 * f + 1] == (int)v) corner = 1;
        else if (a.tri[3 * f + 2] == (int)v) corner = 2;
        for (int d = 0; d < 3; d++) g[d] += a.corner[9 * f + 3 * corner + d];
    }
    for (int d = 0; d < 3; d++) gx[3 * v + d] = g[d];
    if (grho) {
        double gr = 0.0;
        if (a.rho && !a.vclamp[v] && a.grad != 0.0)
            gr = gw * a.va[v] * a.grad * pow(a.rho[v], a.grad - 1.0);
        grho[v] = gr;
    }
}

static inline unsigned nb(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

cudaError_t adjoint_run(const AdjState& a, int metric, int level, double thr, double ratio, double gE,
                        const double* dgE, const double* gC, const uint32_t* sorted, const uint32_t* off,
                        const uint32_t* cnt, double* wsum, double* cent, double* gx, double* grho, cudaStream_t s,
                        Scratch& scratch) {
    adj_face_fwd<<<nb(a.nf), 256, 0, s>>>(a);
    adj_vertex_fwd<<<nb(a.nv), 256, 0, s>>>(a);
    cudaError_t e = sum_f64(a.vw, a.nv, wsum, scratch, s);
    if (e != cudaSuccess) return e;
    adj_clamp<<<nb(a.nv), 256, 0, s>>>(a, wsum, ratio);
    adj_cluster_sums<<<nb((int64_t)a.k * 32), 256, 0, s>>>(a, sorted, off, cnt);
    adj_cluster<<<nb(a.k, 128), 128, 0, s>>>(a, metric, level, thr, gE, dgE, gC, cent);
    g_launches += 6;
    if (gx) {
        adj_face_bwd<<<nb(a.nf), 256, 0, s>>>(a);
        adj_vertex_bwd<<<nb(a.nv), 256, 0, s>>>(a, gx, grho);
        g_launches += 2;
    }
    return cudaGetLastError();
}

size_t adjoint_bytes(int64_t nv, int64_t nf, int k) {
    return sizeof(double) * (size_t)(3 * nf + nf + nf + nv + 6 * nv + nv + (size_t)k * kClStride + 9 * nf + k) + nv;
}

// carves the work buffers out of one allocation
AdjState adjoint_state(void* base, int64_t nv, int64_t nf, int k) {
    AdjState a{};
    double* p = (double*)base;
    a.fn = p; p += 3 * nf;
    a.flen = p; p += nf;
    a.farea = p; p += nf;
    a.va = p; p += nv;
    a.vA = p; p += 6 * nv;
    a.vw = p; p += nv;
    a.cl = p; p += (size_t)k * kClStride;
    a.corner = p; p += 9 * nf;
    a.ek = p; p += k;
    a.vclamp = (unsigned char*)p;
    a.nv = nv; a.nf = nf; a.k = k;
    return a;
}

}  // namespace acvd

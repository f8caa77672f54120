// ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product library includes this file.
//
// Geometry kernels that the reference takes from VTK (not present in this
// environment).  They are restated from the mathematics, not from VTK's source:
//   * triangle area       -- side-length form the reference itself writes in
//                            Common/vtkSurface.cxx:1283 (0.25*sqrt|4ac-(a-b+c)^2|)
//   * plane quadric       -- unit normal n of the triangle, d = -n.x1,
//                            Q = [n;d][n;d]^T  (used by Common/vtkQuadricTools.cxx:66)
//   * symmetric eigen / SVD 3x3 -- cyclic Jacobi rotations (Jacobi 1846; Golub &
//                            Van Loan, "Matrix Computations", sec. 8.5), used by
//                            Common/vtkQuadricTools.cxx:105 through the SVD.
// Both the C++ restatement (acvd_port.cpp) and the VTK shim under oracle/shim call
// these same functions, so the two agree to the last bit wherever the reference's
// own arithmetic is restated faithfully.
#pragma once
#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

namespace rmath {

inline double dist2(const double* a, const double* b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;
}

inline double tri_area(const double* p1, const double* p2, const double* p3) {
    const double a = dist2(p1, p2);
    const double b = dist2(p2, p3);
    const double c = dist2(p3, p1);
    return 0.25 * std::sqrt(std::fabs(4.0 * a * c - (a - b + c) * (a - b + c)));
}

// Unit-normal plane quadric of a triangle; degenerate triangles give a zero quadric.
inline void tri_quadric(const double* x1, const double* x2, const double* x3, double q[4][4]) {
    const double e1[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
    const double e2[3] = {x3[0] - x1[0], x3[1] - x1[1], x3[2] - x1[2]};
    double n[4] = {e1[1] * e2[2] - e1[2] * e2[1],
                   e1[2] * e2[0] - e1[0] * e2[2],
                   e1[0] * e2[1] - e1[1] * e2[0], 0.0};
    const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (len > 0.0) {
        n[0] /= len; n[1] /= len; n[2] /= len;
    } else {
        n[0] = n[1] = n[2] = 0.0;
    }
    n[3] = -(n[0] * x1[0] + n[1] * x1[1] + n[2] * x1[2]);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) q[i][j] = n[i] * n[j];
}

// Unit normal of the triangle (x1, x2, x3) from the cross product
// (x3 - x2) x (x1 - x2) (right-handed in the vertex order); zero for a
// degenerate triangle.  The direction convention is the one the reference's
// vtkTriangle::ComputeNormal callers rely on (VTK >= 9.0, unpinned here).
inline void tri_normal(const double* x1, const double* x2, const double* x3, double n[3]) {
    const double a[3] = {x3[0] - x2[0], x3[1] - x2[1], x3[2] - x2[2]};
    const double b[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
    n[0] = a[1] * b[2] - a[2] * b[1];
    n[1] = a[2] * b[0] - a[0] * b[2];
    n[2] = a[0] * b[1] - a[1] * b[0];
    const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (l != 0.0) { n[0] /= l; n[1] /= l; n[2] /= l; }
}

// Inverse of the n x n matrix a (rows a[i]) by LU decomposition with partial
// pivoting (Doolittle), then one forward / back substitution per unit vector.
// Returns 0 when a pivot is exactly zero (singular), 1 otherwise.  Stands for
// vtkMath::InvertMatrix (VTK >= 9.0, unpinned here).
inline int lu_invert(double** a, double** ai, int n) {
    std::vector<double> lu((size_t)n * n);
    std::vector<int> piv(n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) lu[(size_t)i * n + j] = a[i][j];
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = std::fabs(lu[(size_t)k * n + k]);
        for (int i = k + 1; i < n; i++) {
            const double v = std::fabs(lu[(size_t)i * n + k]);
            if (v > best) { best = v; p = i; }
        }
        if (best == 0.0) return 0;
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < n; j++) std::swap(lu[(size_t)k * n + j], lu[(size_t)p * n + j]);
        const double d = lu[(size_t)k * n + k];
        for (int i = k + 1; i < n; i++) {
            const double f = lu[(size_t)i * n + k] / d;
            lu[(size_t)i * n + k] = f;
            for (int j = k + 1; j < n; j++) lu[(size_t)i * n + j] -= f * lu[(size_t)k * n + j];
        }
    }
    std::vector<double> x(n);
    for (int c = 0; c < n; c++) {
        for (int i = 0; i < n; i++) x[i] = (i == c) ? 1.0 : 0.0;
        for (int k = 0; k < n; k++) if (piv[k] != k) std::swap(x[k], x[piv[k]]);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < i; j++) x[i] -= lu[(size_t)i * n + j] * x[j];
        for (int i = n - 1; i >= 0; i--) {
            for (int j = i + 1; j < n; j++) x[i] -= lu[(size_t)i * n + j] * x[j];
            x[i] /= lu[(size_t)i * n + i];
        }
        for (int i = 0; i < n; i++) ai[i][c] = x[i];
    }
    return 1;
}

// Eigen-decomposition of the symmetric matrix given by the upper triangle of the
// n x n matrix a (a is not modified), by cyclic Jacobi rotations (Jacobi 1846;
// Golub & Van Loan sec. 8.5): eigenvalues w in decreasing order, unit
// eigenvectors in the columns of v.  Returns 1.  Stands for vtkMath::JacobiN
// (VTK >= 9.0, unpinned here); the eigenvector signs are not specified.
inline int jacobi_upper(double** a, int n, double* w, double** v) {
    std::vector<double> m((size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) m[(size_t)i * n + j] = (i <= j) ? a[i][j] : a[j][i];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) v[i][j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += m[(size_t)p * n + q] * m[(size_t)p * n + q];
        if (off == 0.0) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = m[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double theta = (m[(size_t)q * n + q] - m[(size_t)p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double mkp = m[(size_t)k * n + p], mkq = m[(size_t)k * n + q];
                    m[(size_t)k * n + p] = c * mkp - s * mkq;
                    m[(size_t)k * n + q] = s * mkp + c * mkq;
                }
                for (int k = 0; k < n; k++) {
                    const double mpk = m[(size_t)p * n + k], mqk = m[(size_t)q * n + k];
                    m[(size_t)p * n + k] = c * mpk - s * mqk;
                    m[(size_t)q * n + k] = s * mpk + c * mqk;
                }
                m[(size_t)p * n + q] = m[(size_t)q * n + p] = 0.0;
                for (int k = 0; k < n; k++) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; i++) w[i] = m[(size_t)i * n + i];
    // decreasing order (stable selection)
    for (int i = 0; i < n; i++) {
        int b = i;
        for (int j = i + 1; j < n; j++) if (w[j] > w[b]) b = j;
        if (b != i) {
            std::swap(w[i], w[b]);
            for (int k = 0; k < n; k++) std::swap(v[k][i], v[k][b]);
        }
    }
    return 1;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations.
// On return A = V diag(w) V^T, columns of V are the eigenvectors, w sorted by
// decreasing value.  Returns the number of sweeps used.
inline int sym_eig3(const double Ain[3][3], double w[3], double V[3][3]) {
    double a[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { a[i][j] = 0.5 * (Ain[i][j] + Ain[j][i]); V[i][j] = (i == j); }
    int sweep = 0;
    for (; sweep < 64; sweep++) {
        const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        const double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off == 0.0 || off <= 1e-36 * diag) break;
        for (int p = 0; p < 2; p++) {
            for (int q = p + 1; q < 3; q++) {
                const double apq = a[p][q];
                if (apq == 0.0) continue;
                const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0);
                const double s = t * c;
                // A <- J^T A J with J the rotation in the (p,q) plane
                for (int k = 0; k < 3; k++) {
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                a[p][q] = a[q][p] = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
        }
    }
    for (int i = 0; i < 3; i++) w[i] = a[i][i];
    // sort by decreasing eigenvalue (selection sort keeps columns paired)
    for (int i = 0; i < 2; i++) {
        int m = i;
        for (int j = i + 1; j < 3; j++) if (w[j] > w[m]) m = j;
        if (m != i) {
            const double tw = w[i]; w[i] = w[m]; w[m] = tw;
            for (int k = 0; k < 3; k++) { const double tv = V[k][i]; V[k][i] = V[k][m]; V[k][m] = tv; }
        }
    }
    return sweep;
}

// A = U diag(w) VT with w >= 0 sorted by decreasing value.
// Symmetric A: from its eigen-decomposition (w = |lambda|, U = V sign(lambda)).
// General A: V from the eigenvectors of A^T A, U = A V / w (completed to an
// orthonormal frame where w vanishes).
inline void svd3(const double A[3][3], double U[3][3], double w[3], double VT[3][3]) {
    const bool sym = (A[0][1] == A[1][0]) && (A[0][2] == A[2][0]) && (A[1][2] == A[2][1]);
    double V[3][3], lam[3];
    if (sym) {
        sym_eig3(A, lam, V);
        int order[3] = {0, 1, 2};
        for (int i = 0; i < 2; i++)
            for (int j = i + 1; j < 3; j++)
                if (std::fabs(lam[order[j]]) > std::fabs(lam[order[i]])) {
                    const int t = order[i]; order[i] = order[j]; order[j] = t;
                }
        for (int c = 0; c < 3; c++) {
            const int o = order[c];
            w[c] = std::fabs(lam[o]);
            const double sg = lam[o] < 0.0 ? -1.0 : 1.0;
            for (int k = 0; k < 3; k++) { U[k][c] = sg * V[k][o]; VT[c][k] = V[k][o]; }
        }
        return;
    }
    double AtA[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            AtA[i][j] = A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j];
    sym_eig3(AtA, lam, V);
    for (int c = 0; c < 3; c++) {
        w[c] = std::sqrt(lam[c] > 0.0 ? lam[c] : 0.0);
        for (int k = 0; k < 3; k++) VT[c][k] = V[k][c];
    }
    for (int c = 0; c < 3; c++) {
        double u[3];
        for (int k = 0; k < 3; k++) u[k] = A[k][0] * V[0][c] + A[k][1] * V[1][c] + A[k][2] * V[2][c];
        double nrm = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (nrm <= 1e-300) {
            // complete from the previous columns
            double a0[3] = {U[0][0], U[1][0], U[2][0]};
            if (c == 0) { u[0] = 1; u[1] = 0; u[2] = 0; }
            else if (c == 1) {
                const double ref[3] = {std::fabs(a0[0]) < 0.9 ? 1.0 : 0.0, std::fabs(a0[0]) < 0.9 ? 0.0 : 1.0, 0.0};
                u[0] = a0[1] * ref[2] - a0[2] * ref[1];
                u[1] = a0[2] * ref[0] - a0[0] * ref[2];
                u[2] = a0[0] * ref[1] - a0[1] * ref[0];
            } else {
                const double a1[3] = {U[0][1], U[1][1], U[2][1]};
                u[0] = a0[1] * a1[2] - a0[2] * a1[1];
                u[1] = a0[2] * a1[0] - a0[0] * a1[2];
                u[2] = a0[0] * a1[1] - a0[1] * a1[0];
            }
            nrm = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        }
        for (int k = 0; k < 3; k++) U[k][c] = u[k] / nrm;
    }
}

inline void mul33v(const double A[3][3], const double* v, double* out) {
    double t[3];
    for (int i = 0; i < 3; i++) t[i] = A[i][0] * v[0] + A[i][1] * v[1] + A[i][2] * v[2];
    out[0] = t[0]; out[1] = t[1]; out[2] = t[2];
}

inline void mul33(const double A[3][3], const double B[3][3], double C[3][3]) {
    double T[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            T[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) C[i][j] = T[i][j];
}

inline void transpose33(const double A[3][3], double AT[3][3]) {
    double T[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T[i][j] = A[j][i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) AT[i][j] = T[i][j];
}

}  // namespace rmath

// Shared device helpers for the ACVD clustering kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define ACVD_DEV __device__ __forceinline__
#define ACVD_HD __host__ __device__ __forceinline__

namespace acvd {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Compensated float32 accumulation ("double-float"): value = hi + lo with
// |lo| <= ulp(hi)/2.  Additions use Knuth's TwoSum; products of two floats are
// split exactly with an FMA (TwoProd).  About 48 significant bits, float ALUs only.
// ---------------------------------------------------------------------------
struct df { float hi, lo; };

ACVD_DEV df df_make(float x) { return {x, 0.0f}; }

#ifdef ACVD_PLAIN_FP32
// The plain form (a second build of the clustering kernels, libacvd_gb300_plain):
// every double-float operation keeps only its rounded float32 leading part, so
// cluster sums, incremental records and relaxed-step folds are plain float32
// arithmetic.  It exists to measure what the compensation buys.
ACVD_DEV df df_add(df x, df y) { return {__fadd_rn(x.hi, y.hi), 0.0f}; }
ACVD_DEV df df_add_f(df x, float y) { return {__fadd_rn(x.hi, y), 0.0f}; }
ACVD_DEV df df_neg(df x) { return {-x.hi, 0.0f}; }
ACVD_DEV df two_prod(float a, float b) { return {__fmul_rn(a, b), 0.0f}; }
ACVD_DEV double df_to_d(df x) { return (double)x.hi; }
ACVD_DEV df df_renorm(float s, float e) { return {__fadd_rn(s, e), 0.0f}; }
ACVD_DEV df df_sub(df x, df y) { return {__fsub_rn(x.hi, y.hi), 0.0f}; }
ACVD_DEV df df_mul(df x, df y) { return {__fmul_rn(x.hi, y.hi), 0.0f}; }
ACVD_DEV df df_mul_f(df x, float y) { return {__fmul_rn(x.hi, y), 0.0f}; }
ACVD_DEV df df_div(df x, df y) { return {__fdiv_rn(x.hi, y.hi), 0.0f}; }
ACVD_DEV df df_from_d(double v) { return {__double2float_rn(v), 0.0f}; }
#else

ACVD_DEV void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

ACVD_DEV void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// x += y (both double-float)
ACVD_DEV df df_add(df x, df y) {
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    float h, l;
    fast_two_sum(s, e, h, l);
    return {h, l};
}

ACVD_DEV df df_add_f(df x, float y) {
    float s, e;
    two_sum(x.hi, y, s, e);
    e = __fadd_rn(e, x.lo);
    float h, l;
    fast_two_sum(s, e, h, l);
    return {h, l};
}

ACVD_DEV df df_neg(df x) { return {-x.hi, -x.lo}; }

// exact product of two floats as a double-float
ACVD_DEV df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return {p, e};
}

ACVD_DEV double df_to_d(df x) { return (double)x.hi + (double)x.lo; }

ACVD_DEV df df_renorm(float s, float e) {
    float h, l;
    fast_two_sum(s, e, h, l);
    return {h, l};
}

ACVD_DEV df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

// Products and quotient of double-floats (Dekker 1971, "A floating-point
// technique for extending the available precision"; the same steps as Hida, Li
// and Bailey's double-double library): one exact TwoProd of the leading parts
// plus the cross terms, renormalised.  About 2^-47 relative error.
ACVD_DEV df df_mul(df x, df y) {
    df p = two_prod(x.hi, y.hi);
    p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
    p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
    return df_renorm(p.hi, p.lo);
}

ACVD_DEV df df_mul_f(df x, float y) {
    df p = two_prod(x.hi, y);
    p.lo = __fmaf_rn(x.lo, y, p.lo);
    return df_renorm(p.hi, p.lo);
}

// x / y: a float quotient, then one correction from the remainder x - y q1
ACVD_DEV df df_div(df x, df y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const df r = df_sub(x, df_mul_f(y, q1));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    return df_renorm(q1, q2);
}



ACVD_DEV df df_from_d(double v) {
    const float h = __double2float_rn(v);
    const float l = __double2float_rn(v - (double)h);
    return {h, l};
}
#endif  // ACVD_PLAIN_FP32

// ---------------------------------------------------------------------------
// Claim words: [8-bit epoch (descending)][30-bit priority][26-bit item slot].
// Smaller is better, so atomicMin keeps the best candidate of the newest step
// without a reset pass between steps.
// ---------------------------------------------------------------------------
constexpr int kEpochBits = 8;
constexpr int kPrioBits = 30;
constexpr int kSlotBits = 26;
constexpr unsigned long long kClaimEmpty = ~0ull;

ACVD_HD unsigned long long make_claim(unsigned epoch, unsigned prio, unsigned slot) {
    const unsigned long long e = (unsigned long long)(255u - (epoch & 255u));
    return (e << (kPrioBits + kSlotBits)) |
           ((unsigned long long)(prio & ((1u << kPrioBits) - 1u)) << kSlotBits) |
           (unsigned long long)(slot & ((1u << kSlotBits) - 1u));
}

// Priority of an energy decrease dE < 0: larger |dE| gives a smaller priority.
ACVD_DEV unsigned prio_of_delta(float dE) {
    const unsigned mag = __float_as_uint(dE) & 0x7fffffffu;   // |dE| bits, monotone in |dE|
    const unsigned q = mag >> 1;                               // 30 bits
    return ((1u << kPrioBits) - 1u) - q;
}

// ---------------------------------------------------------------------------
// Small symmetric 3x3 eigen-solver by cyclic Jacobi rotations (Jacobi 1846;
// Golub & Van Loan, Matrix Computations, sec. 8.5).  a = {a00,a01,a02,a11,a12,a22}.
// On return w holds the eigenvalues and V (columns) the eigenvectors.
// ---------------------------------------------------------------------------
template <typename T>
ACVD_DEV void jacobi_eig3(const T a6[6], T w[3], T V[3][3], int max_sweeps) {
    T A[3][3] = {{a6[0], a6[1], a6[2]}, {a6[1], a6[3], a6[4]}, {a6[2], a6[4], a6[5]}};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) V[i][j] = (i == j) ? T(1) : T(0);
    const T tiny = sizeof(T) == 4 ? T(1e-14) : T(1e-30);
    for (int s = 0; s < max_sweeps; s++) {
        const T off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        const T dg = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (!(off > tiny * dg)) break;
#pragma unroll
        for (int pq = 0; pq < 3; pq++) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const T apq = A[p][q];
            if (apq == T(0)) continue;
            const T theta = (A[q][q] - A[p][p]) / (T(2) * apq);
            const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
            const T c = T(1) / sqrt(t * t + T(1));
            const T sn = t * c;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T akp = A[k][p], akq = A[k][q];
                A[k][p] = c * akp - sn * akq;
                A[k][q] = sn * akp + c * akq;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T apk = A[p][k], aqk = A[q][k];
                A[p][k] = c * apk - sn * aqk;
                A[q][k] = sn * apk + c * aqk;
            }
            A[p][q] = A[q][p] = T(0);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T vkp = V[k][p], vkq = V[k][q];
                V[k][p] = c * vkp - sn * vkq;
                V[k][q] = sn * vkp + c * vkq;
            }
        }
    }
    w[0] = A[0][0]; w[1] = A[1][1]; w[2] = A[2][2];
}

// Thresholded pseudo-inverse applied to r, as the reference's quadric vertex
// placement does (Common/vtkQuadricTools.cxx:83-163): eigenvalues are taken in
// decreasing |lambda|; at most `level` of them, and only those with
// |lambda| / max|lambda| > thr, are inverted.  Returns pinv(A) r in d and the
// rank deficiency.
// One eigenpair: |lambda|, lambda, eigenvector.
template <typename T>
struct EigPair {
    T a, w, v0, v1, v2;
};

// Swaps x and y when x.a < y.a (strictly), so that equal magnitudes keep their order.
template <typename T>
ACVD_DEV void eig_order(EigPair<T>& x, EigPair<T>& y) {
    if (x.a < y.a) {
        const EigPair<T> t = x;
        x = y;
        y = t;
    }
}

template <typename T>
ACVD_DEV int pinv_apply(const T a6[6], const T r[3], T d[3], int level, T thr, int max_sweeps) {
    T w[3], V[3][3];
    jacobi_eig3<T>(a6, w, V, max_sweeps);
    // the eigenpairs in decreasing |lambda|, equal magnitudes in index order (a stable
    // three-element sorting network on registers)
    EigPair<T> e0 = {fabs(w[0]), w[0], V[0][0], V[1][0], V[2][0]};
    EigPair<T> e1 = {fabs(w[1]), w[1], V[0][1], V[1][1], V[2][1]};
    EigPair<T> e2 = {fabs(w[2]), w[2], V[0][2], V[1][2], V[2][2]};
    eig_order(e0, e1);
    eig_order(e1, e2);
    eig_order(e0, e1);
    const T mx = e0.a;
    d[0] = d[1] = d[2] = T(0);
    int used = 0, rank_def = 0;
    auto take = [&](const EigPair<T>& e) {
        const bool keep = (mx > T(0)) && (e.a > thr * mx) && (used < level);
        if (keep) {
            const T proj = (e.v0 * r[0] + e.v1 * r[1] + e.v2 * r[2]) / e.w;
            d[0] += proj * e.v0;
            d[1] += proj * e.v1;
            d[2] += proj * e.v2;
            used++;
        } else {
            rank_def++;
        }
    };
    take(e0);
    take(e1);
    take(e2);
    return rank_def;
}

ACVD_DEV float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

}  // namespace acvd

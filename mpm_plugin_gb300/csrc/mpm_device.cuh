// Device-side math of the MLS-MPM substep: 3x3 SVD, quadratic B-spline weights, constitutive models and
// return mappings, mesh closest-point queries. Each function names the reference code it computes the
// same result as (mpm_core/backends/warp/kernels.py, colliders.py).
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "mpm_types.h"

// The math below also compiles for the host (tests check the SVD's accuracy on the CPU).
#define MPM_HD __host__ __device__ __forceinline__

namespace mpm {

#ifndef __CUDA_ARCH__
using std::isfinite;
#endif

// Arithmetic with every operation rounded on its own (no fused multiply-add), for the values whose last bits
// decide a discrete choice or are magnified downstream (the collider pose, a grid node's position, the local
// query point, FP64 distances that break near-ties between mesh faces, the closest point, normal and contact
// response of a collider query): these follow the reference's operation order.
#ifdef __CUDA_ARCH__
MPM_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
MPM_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
MPM_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
MPM_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
MPM_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
MPM_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
MPM_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
MPM_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
MPM_HD float fsqrt(float a) { return __fsqrt_rn(a); }
#else  // host: a volatile store keeps the compiler from fusing the operation into a multiply-add
MPM_HD float fadd(float a, float b) { volatile float r = a + b; return r; }
MPM_HD float fsub(float a, float b) { volatile float r = a - b; return r; }
MPM_HD float fmul(float a, float b) { volatile float r = a * b; return r; }
MPM_HD float fdiv(float a, float b) { volatile float r = a / b; return r; }
MPM_HD double dadd(double a, double b) { volatile double r = a + b; return r; }
MPM_HD double dsub(double a, double b) { volatile double r = a - b; return r; }
MPM_HD double dmul(double a, double b) { volatile double r = a * b; return r; }
MPM_HD double ddiv(double a, double b) { volatile double r = a / b; return r; }
MPM_HD float fsqrt(float a) { volatile float r = sqrtf(a); return r; }
#endif
// a0 b0 + a1 b1 + a2 b2, left to right, each operation rounded on its own
MPM_HD float fdot3(const float a[3], const float b[3]) {
    return fadd(fadd(fmul(a[0], b[0]), fmul(a[1], b[1])), fmul(a[2], b[2]));
}

// ---------------------------------------------------------------------------------------------------------
// 3x3 SVD with the convention of Warp's svd3 (called at kernels.py:35,57,252): U and V proper rotations,
// singular values in decreasing order, the sign of det(A) carried by the last one.
//
// Method: cyclic Jacobi eigen-decomposition of a symmetric 3x3 with exact rotation angles (the Numerical
// Recipes 11.1 update) for V, then a Givens QR of A V for U (McAdams et al. 2011 use this split, with
// approximate angles). The FP32 instance reports how far its QR factor is from diagonal; the rare lanes
// that did not converge are redone in FP64.
// ---------------------------------------------------------------------------------------------------------
template <typename T>
MPM_HD T rsqrt_t(T x);
#ifdef __CUDA_ARCH__
template <>
MPM_HD float rsqrt_t<float>(float x) { return rsqrtf(x); }
template <>
MPM_HD double rsqrt_t<double>(double x) { return rsqrt(x); }
#else
template <>
MPM_HD float rsqrt_t<float>(float x) { return 1.0f / sqrtf(x); }
template <>
MPM_HD double rsqrt_t<double>(double x) { return 1.0 / sqrt(x); }
#endif

template <typename T>
MPM_HD T sqrt_t(T x) { return sqrt(x); }

// Quotient and square root inside a Jacobi rotation. The rotation stays orthogonal whatever the rounding of
// its angle (c = 1 / sqrt(1 + t^2), s = t c), so FP32 takes the hardware approximations (2 ulp) there;
// FP64 keeps IEEE operations.
template <typename T>
MPM_HD T rot_div(T a, T b) { return a / b; }
template <typename T>
MPM_HD T rot_sqrt(T x) { return sqrt_t(x); }  // x >= 1
#ifdef __CUDA_ARCH__
template <>
MPM_HD float rot_div<float>(float a, float b) { return __fdividef(a, b); }
template <>
MPM_HD float rot_sqrt<float>(float x) { return x * rsqrtf(x); }
#endif

template <typename T>
MPM_HD void jacobi_rotate(T S[3][3], T V[3][3], int p, int q) {
    const int r = 3 - p - q;
    T apq = S[p][q];
    // an off-diagonal this small is already negligible against the 4e-6 convergence bound (and would
    // overflow the quotient); NaN passes on to the convergence check
    if (fabs(apq) < T(1e-30)) return;
    T zeta = rot_div<T>(S[q][q] - S[p][p], T(2) * apq);
    T az = fabs(zeta);
    // t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)); for huge |zeta| the square would overflow, t -> 1/(2 zeta)
    T t = az > T(1e18) ? rot_div<T>(T(0.5), zeta)
                       : rot_div<T>(copysign(T(1), zeta), az + rot_sqrt<T>(T(1) + zeta * zeta));
    T c = rsqrt_t(T(1) + t * t);
    T s = t * c;
    S[p][p] -= t * apq;
    S[q][q] += t * apq;
    S[p][q] = S[q][p] = T(0);
    T srp = S[r][p], srq = S[r][q];
    S[r][p] = S[p][r] = c * srp - s * srq;
    S[r][q] = S[q][r] = s * srp + c * srq;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T vp = V[i][p], vq = V[i][q];
        V[i][p] = c * vp - s * vq;
        V[i][q] = s * vp + c * vq;
    }
}

// Givens rotation zeroing B[b][col] against B[a][col]; accumulates U <- U G^T.
template <typename T>
MPM_HD void givens_qr_step(T B[3][3], T U[3][3], int a, int b, int col) {
    T x = B[a][col], y = B[b][col];
    T rr = x * x + y * y;
    T c = T(1), s = T(0);
    if (rr > T(0)) {
        T inv = rsqrt_t(rr);
        c = x * inv;
        s = y * inv;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        T ba = B[a][j], bb = B[b][j];
        B[a][j] = c * ba + s * bb;
        B[b][j] = -s * ba + c * bb;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T ua = U[i][a], ub = U[i][b];
        U[i][a] = c * ua + s * ub;
        U[i][b] = -s * ua + c * ub;
    }
}

template <typename T>
MPM_HD void swap_cols(T M[3][3], int a, int b, bool negate) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T t = M[i][a];
        M[i][a] = negate ? -M[i][b] : M[i][b];
        M[i][b] = t;
    }
}

// An off-diagonal of E = A^T A - I below this after two Jacobi sweeps moves the reconstructed U diag(sigma)
// V^T by about half of it (sigma ~ 1), below an FP32 ulp of 1, and the QR factor's off-diagonals stay far
// inside the 4e-6 convergence bound: no further sweep runs for such a lane.
constexpr float kSweepSkip = 1.0e-8f;
// ... or below this fraction of E's largest diagonal entry (about three FP32 ulps of it).
constexpr float kSweepSkipRel = 4.0e-7f;
// Sweeps after the first two, at most, for a lane whose E is not yet diagonal to kSweepSkip.
constexpr int kMaxExtraSweeps = 6;

// ---------------------------------------------------------------------------------------------------------
// SVD in deviation form, for the MPM regime F ~ I. The eigenvalues of E = A^T A - I, formed as
// G + G^T + G^T G from G = A - I (exact in FP32 near I), give d = sigma - 1 to full relative accuracy,
// so strains of 1e-4 keep ~7 significant digits where sigma itself would keep 3 (singular values below 0.5
// come from the QR diagonal instead, where sqrt(1 + e) would cancel). V: Jacobi eigenvectors of E;
// U: Givens QR of A V (proper rotation; the QR factor's last diagonal carries sign(det A)).
// Returns the largest off-diagonal of the QR factor relative to sigma_0 (a convergence measure).
// kAdaptive: two sweeps, then further sweeps (one copy of the code, a loop) while an off-diagonal of E is
// above kSweepSkip, at most kMaxExtraSweeps; SWEEPS is then unused. The lane's own E decides, so a
// particle's result does not depend on its neighbours in the warp.
// ---------------------------------------------------------------------------------------------------------
// kWarm: the sweeps start from the basis V0 (a rotation: the previous substep's V), on V0^T E V0, which is
// nearly diagonal when the particle deformed little since; one sweep is then mandatory instead of two.
template <typename T, int SWEEPS, bool kAdaptive = false, bool kWarm = false>
MPM_HD T svd3_dev_core(const T A[3][3], T U[3][3], T sig[3], T d[3], T V[3][3], const T (*V0)[3] = nullptr) {
    T G[3][3], E[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) G[i][j] = A[i][j] - (i == j ? T(1) : T(0));
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            E[i][j] = G[i][j] + G[j][i] + (G[0][i] * G[0][j] + G[1][i] * G[1][j] + G[2][i] * G[2][j]);
            V[i][j] = i == j ? T(1) : T(0);
            U[i][j] = i == j ? T(1) : T(0);
        }
    if constexpr (kWarm) {  // E <- V0^T E V0 (symmetric), V <- V0
        T W[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) W[i][j] = E[i][0] * V0[0][j] + E[i][1] * V0[1][j] + E[i][2] * V0[2][j];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                E[i][j] = V0[0][i] * W[0][j] + V0[1][i] * W[1][j] + V0[2][i] * W[2][j];
                E[j][i] = E[i][j];
            }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) V[i][j] = V0[i][j];
    }
#pragma unroll
    for (int sw = 0; sw < (kAdaptive ? (kWarm ? 1 : 2) : SWEEPS); ++sw) {
        jacobi_rotate(E, V, 0, 1);
        jacobi_rotate(E, V, 0, 2);
        jacobi_rotate(E, V, 1, 2);
    }
    if constexpr (kAdaptive) {
        // the bound grows with E where kSweepSkip is below its rounding (a strain of 0.2 keeps off-diagonals of
        // a few 1e-8 whatever the sweeps do)
        const T skip = fmax(T(kSweepSkip), T(kSweepSkipRel) * fmax(fmax(fabs(E[0][0]), fabs(E[1][1])), fabs(E[2][2])));
#pragma unroll 1
        for (int sw = 0; sw < kMaxExtraSweeps && fmax(fmax(fabs(E[0][1]), fabs(E[0][2])), fabs(E[1][2])) > skip; ++sw) {
            jacobi_rotate(E, V, 0, 1);
            jacobi_rotate(E, V, 0, 2);
            jacobi_rotate(E, V, 1, 2);
        }
    }
    T e0 = E[0][0], e1 = E[1][1], e2 = E[2][2];
    // descending eigenvalues; a swap negates one column so det(V) stays +1
    if (e0 < e1) { swap_cols(V, 0, 1, true); T t = e0; e0 = e1; e1 = t; }
    if (e0 < e2) { swap_cols(V, 0, 2, true); T t = e0; e0 = e2; e2 = t; }
    if (e1 < e2) { swap_cols(V, 1, 2, true); T t = e1; e1 = e2; e2 = t; }
    const T e[3] = {e0, e1, e2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T r = sqrt_t(fmax(T(1) + e[i], T(0)));
        d[i] = e[i] / (T(1) + r);  // sigma - 1 without cancellation
        sig[i] = T(1) + d[i];
    }
    T B[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B[i][j] = A[i][0] * V[0][j] + A[i][1] * V[1][j] + A[i][2] * V[2][j];
    givens_qr_step(B, U, 0, 1, 0);
    givens_qr_step(B, U, 0, 2, 0);
    givens_qr_step(B, U, 1, 2, 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (T(1) + e[i] < T(0.25)) {  // sigma < 0.5: sqrt(1 + e) cancels, the QR diagonal is accurate
            sig[i] = fabs(B[i][i]);
            d[i] = sig[i] - T(1);
        }
    if (B[2][2] < T(0)) {  // inverted: the last singular value carries the sign of det(A)
        sig[2] = -sig[2];
        d[2] = sig[2] - T(1);
    }
    T off = fmax(fmax(fabs(B[0][1]), fabs(B[0][2])), fabs(B[1][2]));
    T scale = fabs(sig[0]);
    return scale > T(0) ? off / scale : T(0);
}

// FP32 deviation-form SVD: two cyclic Jacobi sweeps (one when started from V0, the previous basis), then
// more (up to eight in all) while E is not diagonal to kSweepSkip. kFp64: lanes whose sweeps did not
// diagonalise E to 4e-6 (relative to sigma_0) are redone in FP64 (from scratch); either way they are counted
// when a counter is given. The default G2P builds take kFp64 = false: the
// FP64 code in line with the FP32 path made the compiler spill the FP32 path's registers (152 against 32
// bytes of spill stores at 80 registers; G2P 35.3 against 31.2 us on the mixed workload, measured) although
// no lane took it there. Measured on the mixed workload with a fixed sweep count: three sweeps left no lane
// unconverged over thousands of substeps, two sweeps for every lane left millions within three frames.
template <bool kFp64 = true>
MPM_HD void svd3(const float A[3][3], float U[3][3], float sig[3], float d[3], float V[3][3],
                 unsigned int* fp64_lanes, const float (*V0)[3] = nullptr) {
    const float off = V0 ? svd3_dev_core<float, 3, true, true>(A, U, sig, d, V, V0)
                         : svd3_dev_core<float, 3, true>(A, U, sig, d, V);
    if (!kFp64) {
        if (!(off <= 4e-6f) && fp64_lanes) {  // NaN input stays NaN
#ifdef __CUDA_ARCH__
            atomicAdd(fp64_lanes, 1u);
#else
            *fp64_lanes += 1u;
#endif
        }
        return;
    }
    if (!(off <= 4e-6f)) {  // also taken for NaN input, which then stays NaN
        double Ad[3][3], Ud[3][3], sd[3], dd[3], Vd[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Ad[i][j] = A[i][j];
        svd3_dev_core<double, 8>(Ad, Ud, sd, dd, Vd);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            sig[i] = (float)sd[i];
            d[i] = (float)dd[i];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                U[i][j] = (float)Ud[i][j];
                V[i][j] = (float)Vd[i][j];
            }
        }
#ifdef __CUDA_ARCH__
        if (fp64_lanes) atomicAdd(fp64_lanes, 1u);
#else
        if (fp64_lanes) *fp64_lanes += 1u;
#endif
    }
}

// A rotation matrix as a unit quaternion (x, y, z, w), by Shepperd's method (1978): the square root is taken
// of the largest of 1 + trace and the 1 + 2 R_ii - trace, so it never cancels.
MPM_HD void rotation_to_quat(const float R[3][3], float q[4]) {
    const float tr = R[0][0] + R[1][1] + R[2][2];
    if (tr > 0.0f) {
        const float s = 2.0f * sqrtf(1.0f + tr), inv = 1.0f / s;
        q[3] = 0.25f * s;
        q[0] = (R[2][1] - R[1][2]) * inv;
        q[1] = (R[0][2] - R[2][0]) * inv;
        q[2] = (R[1][0] - R[0][1]) * inv;
    } else if (R[0][0] > R[1][1] && R[0][0] > R[2][2]) {
        const float s = 2.0f * sqrtf(1.0f + R[0][0] - R[1][1] - R[2][2]), inv = 1.0f / s;
        q[3] = (R[2][1] - R[1][2]) * inv;
        q[0] = 0.25f * s;
        q[1] = (R[0][1] + R[1][0]) * inv;
        q[2] = (R[0][2] + R[2][0]) * inv;
    } else if (R[1][1] > R[2][2]) {
        const float s = 2.0f * sqrtf(1.0f + R[1][1] - R[0][0] - R[2][2]), inv = 1.0f / s;
        q[3] = (R[0][2] - R[2][0]) * inv;
        q[0] = (R[0][1] + R[1][0]) * inv;
        q[1] = 0.25f * s;
        q[2] = (R[1][2] + R[2][1]) * inv;
    } else {
        const float s = 2.0f * sqrtf(1.0f + R[2][2] - R[0][0] - R[1][1]), inv = 1.0f / s;
        q[3] = (R[1][0] - R[0][1]) * inv;
        q[0] = (R[0][2] + R[2][0]) * inv;
        q[1] = (R[1][2] + R[2][1]) * inv;
        q[2] = 0.25f * s;
    }
}

// The rotation of a quaternion (x, y, z, w), normalised first; the identity for one that is not finite or
// far from unit length (a particle whose basis was never set, or a blown-up one).
MPM_HD void quat_to_rotation(const float q[4], float R[3][3]) {
    const float n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (!(n2 > 0.5f && n2 < 2.0f)) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) R[i][j] = i == j ? 1.0f : 0.0f;
        return;
    }
    const float k = 2.0f / n2;
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    R[0][0] = 1.0f - k * (y * y + z * z);
    R[0][1] = k * (x * y - z * w);
    R[0][2] = k * (x * z + y * w);
    R[1][0] = k * (x * y + z * w);
    R[1][1] = 1.0f - k * (x * x + z * z);
    R[1][2] = k * (y * z - x * w);
    R[2][0] = k * (x * z - y * w);
    R[2][1] = k * (y * z + x * w);
    R[2][2] = 1.0f - k * (x * x + y * y);
}

// ---------------------------------------------------------------------------------------------------------
// Quadratic B-spline weights and stencil base: kernels.py:16-27
// ---------------------------------------------------------------------------------------------------------
// Stencil base along one axis: floor(xp - 0.5) (kernels.py:25-27). Returns false when the 3-node stencil
// would leave the padded grid, which also catches NaN and inf positions; such a particle neither scatters
// nor gathers, so a blown-up particle can never address memory outside the grid.
MPM_HD bool stencil_axis(float xp, int dims, int* base, float* fx) {
    float b = floorf(xp - 0.5f);
    bool ok = b >= 0.0f && b <= (float)(dims - 3);
    *base = ok ? (int)b : 0;
    *fx = xp - b;
    return ok;
}

MPM_HD void bspline_weights(float fx, float w[3]) {
    w[0] = 0.5f * (1.5f - fx) * (1.5f - fx);
    w[1] = 0.75f - (fx - 1.0f) * (fx - 1.0f);
    w[2] = 0.5f * (fx - 0.5f) * (fx - 0.5f);
}

// ---------------------------------------------------------------------------------------------------------
// Kirchhoff stress, written on the left singular basis so no F - R cancellation occurs:
//   fixed-corotated (kernels.py:30-38): 2 mu (F - R) F^T + lam J (J - 1) I = U diag(2 mu (s-1) s + lam J (J-1)) U^T
//   Hencky / St. Venant-Kirchhoff (kernels.py:51-60): U diag(2 mu eps + lam tr eps) U^T, eps = log max(s, 1e-4)
// ---------------------------------------------------------------------------------------------------------
// Elementary functions of either precision (the float versions are the single-precision calls).
MPM_HD float log1p_t(float x) { return log1pf(x); }
MPM_HD double log1p_t(double x) { return log1p(x); }
MPM_HD float expm1_t(float x) { return expm1f(x); }
MPM_HD double expm1_t(double x) { return expm1(x); }
MPM_HD float log_t(float x) { return logf(x); }
MPM_HD double log_t(double x) { return log(x); }
MPM_HD float exp_t(float x) { return expf(x); }
MPM_HD double exp_t(double x) { return exp(x); }
MPM_HD float min_t(float a, float b) { return fminf(a, b); }
MPM_HD double min_t(double a, double b) { return fmin(a, b); }
MPM_HD float max_t(float a, float b) { return fmaxf(a, b); }
MPM_HD double max_t(double a, double b) { return fmax(a, b); }

template <typename T>
MPM_HD T jm1(const T d[3]) {  // J - 1 = prod(1 + d) - 1, expanded so small strains keep their digits
    return d[0] + d[1] + d[2] + (d[0] * d[1] + d[0] * d[2] + d[1] * d[2]) + d[0] * d[1] * d[2];
}

template <typename T>
MPM_HD void sym_from_diag(const T U[3][3], const T g[3], T tau[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tau[i][j] = U[i][0] * g[0] * U[j][0] + U[i][1] * g[1] * U[j][1] + U[i][2] * g[2] * U[j][2];
}

// Principal Kirchhoff stresses of the fixed-corotated energy (kernels.py:30-38) from the singular values sig
// and their deviations d = sig - 1: 2 mu (sig - 1) sig + lam (J - 1) J.
template <typename T>
MPM_HD void corotated_principal(T mu, T lam, const T sig[3], const T d[3], T g[3]) {
    T Jm1 = jm1(d);
    T iso = lam * (T(1) + Jm1) * Jm1;
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] = T(2) * mu * d[i] * sig[i] + iso;
}

template <typename T>
MPM_HD T safe_log_dev(T s, T d) {  // log(max(s, 1e-4)) from d = s - 1 (kernels.py:41-43)
    return s > T(1.0e-4f) ? log1p_t(d) : log_t(T(1.0e-4f));
}

// Principal Kirchhoff stresses of the Hencky (logarithmic) energy (kernels.py:51-60): 2 mu e + lam tr(e).
template <typename T>
MPM_HD void hencky_principal(T mu, T lam, const T sig[3], const T d[3], T g[3]) {
    T e0 = safe_log_dev(sig[0], d[0]), e1 = safe_log_dev(sig[1], d[1]), e2 = safe_log_dev(sig[2], d[2]);
    T tr = e0 + e1 + e2;
    T two_mu = T(2) * mu;
    g[0] = two_mu * e0 + lam * tr;
    g[1] = two_mu * e1 + lam * tr;
    g[2] = two_mu * e2 + lam * tr;
}

MPM_HD void fixed_corotated_tau(const float F[3][3], float mu, float lam, float tau[3][3], unsigned int* fp64) {
    float U[3][3], sig[3], d[3], V[3][3], g[3];
    svd3(F, U, sig, d, V, fp64);
    corotated_principal(mu, lam, sig, d, g);
    sym_from_diag(U, g, tau);
}

MPM_HD void hencky_tau(const float F[3][3], float mu, float lam, float tau[3][3], unsigned int* fp64) {
    float U[3][3], sig[3], d[3], V[3][3], g[3];
    svd3(F, U, sig, d, V, fp64);
    hencky_principal(mu, lam, sig, d, g);
    sym_from_diag(U, g, tau);
}

// ---------------------------------------------------------------------------------------------------------
// Return mappings on singular values: von Mises (kernels.py:63-72), Drucker-Prager after Klar et al. 2016
// (kernels.py:75-89) and the snow clamp of Stomakhin et al. 2013 (kernels.py:258-262). Each returns the
// change of the singular values, delta = new - old, computed without cancellation; the caller applies
// F <- F + U diag(delta) V^T, which equals U diag(new) V^T exactly when the SVD is exact and leaves F
// untouched (no reconstruction round-off) when nothing is projected. Returns false when delta == 0.
// Written for either precision: FP32 for the bulk, FP64 for the optional redo of marginal decisions.
// ---------------------------------------------------------------------------------------------------------
template <typename T>
MPM_HD bool project_von_mises(const T sig[3], const T d[3], T mu, T yield_stress, T delta[3]) {
    T e[3] = {safe_log_dev(sig[0], d[0]), safe_log_dev(sig[1], d[1]), safe_log_dev(sig[2], d[2])};
    T third = (e[0] + e[1] + e[2]) / T(3);
    T dev[3] = {e[0] - third, e[1] - third, e[2] - third};
    T n = sqrt_t(dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]);
    T limit = yield_stress / (T(2) * mu);
    if (!(n > limit)) return false;
    T f = limit / n;
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = expm1_t(third + dev[i] * f) - d[i];
    return true;
}

// A return-mapping decision is marginal when an FP32 evaluation may take it differently from an exact one
// AND the two outcomes differ by more than the FP32 rounding of the result; the FP32 call reports it, and
// the G2P build with the FP64 option redoes those lanes in FP64.
//
// Only the Drucker-Prager separation test is such a decision: tr eps >= 0 sends the log singular values eps
// to 0, just below it they stay or go towards the cone, a jump of at most |eps|_1 (the deviatoric part, n,
// is no larger). It is marginal when |tr eps| lies within kMarginalRel of |eps|_1 (about eight FP32 ulps of
// the terms summed; in the deviation form eps keeps full relative accuracy) and |eps|_1 exceeds
// kMarginalFloor (eight FP32 ulps of 1: below it the jump is at the rounding of the stored F). The cone and
// the snow clamps are continuous in the singular values, and so is the cone projection where n is tiny (the
// projection then moves eps by at most n): a flipped decision there changes the result by rounding.
// Measured on the 256^3 pile: flagging the cone and snow bounds, and then the separation test without the
// floor (settled grains whose strains are a few ulps, where opposite ulps cancel in tr exactly), each marked
// 5 % of the lanes, doubled G2P's time through warp divergence and moved the error against the FP64 oracle
// by nothing.
constexpr float kMarginalRel = 1.0e-6f;
constexpr float kMarginalFloor = 1.0e-6f;

// marginal (optional): set when the separation decision is marginal (above).
template <typename T>
MPM_HD bool project_drucker_prager(const T sig[3], const T d[3], T mu, T lam, T alpha, T delta[3],
                                   bool* marginal = nullptr) {
    T e[3] = {safe_log_dev(sig[0], d[0]), safe_log_dev(sig[1], d[1]), safe_log_dev(sig[2], d[2])};
    T tr = e[0] + e[1] + e[2];
    const T size = fabs(e[0]) + fabs(e[1]) + fabs(e[2]);
    // (strict comparisons: an undeformed particle, all e exactly 0, has no decision to make)
    if (marginal) *marginal = fabs(tr) < T(kMarginalRel) * size && size > T(kMarginalFloor);
    if (tr >= T(0)) {  // separation: stress-free, singular values back to 1
#pragma unroll
        for (int i = 0; i < 3; ++i) delta[i] = -d[i];
        return true;
    }
    T third = tr / T(3);
    T dev[3] = {e[0] - third, e[1] - third, e[2] - third};
    T n = sqrt_t(dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2]);
    const T cone = (T(3) * lam + T(2) * mu) / (T(2) * mu) * tr * alpha;
    if (n < T(1.0e-10f)) return false;
    T dgamma = n + cone;
    if (dgamma <= T(0)) return false;
    T f = dgamma / n;
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = expm1_t(e[i] - dev[i] * f) - d[i];
    return true;
}

// marginal (optional): always false, the clamp being continuous (kept for the callers' symmetry).
template <typename T>
MPM_HD bool project_snow(const T sig[3], const T d[3], T clamp_lo, T clamp_hi, T delta[3], T* jp_ratio,
                         bool* marginal = nullptr) {
    bool any = false;
    T num = T(1), den = T(1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T ns = min_t(max_t(sig[i], clamp_lo), clamp_hi);
        delta[i] = ns == sig[i] ? T(0) : (ns - T(1)) - d[i];
        any |= delta[i] != T(0);
        num *= sig[i];
        den *= ns;
    }
    *jp_ratio = num / den;
    if (marginal) *marginal = false;
    return any;
}

// ---------------------------------------------------------------------------------------------------------
// Mesh queries: exact closest point on a triangle (Ericson, Real-Time Collision Detection 5.1.5) over a
// BVH in the collider's local space; inside/outside from the angle-weighted pseudonormal of the closest
// feature (Baerentzen & Aanaes 2005). Same meaning as Warp's mesh_query_point_sign_normal (colliders.py:50).
// ---------------------------------------------------------------------------------------------------------
// region: 0 face, 1..3 vertex a..c, 4 edge ab, 5 edge bc, 6 edge ca
template <typename T>
MPM_HD void closest_on_triangle(const T p[3], const T a[3], const T b[3], const T c[3], T bary[3], int* region) {
    T ab[3], ac[3], ap[3], bp[3], cp[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        ab[i] = b[i] - a[i]; ac[i] = c[i] - a[i]; ap[i] = p[i] - a[i]; bp[i] = p[i] - b[i]; cp[i] = p[i] - c[i];
    }
    T d1 = ab[0] * ap[0] + ab[1] * ap[1] + ab[2] * ap[2];
    T d2 = ac[0] * ap[0] + ac[1] * ap[1] + ac[2] * ap[2];
    T d3 = ab[0] * bp[0] + ab[1] * bp[1] + ab[2] * bp[2];
    T d4 = ac[0] * bp[0] + ac[1] * bp[1] + ac[2] * bp[2];
    T d5 = ab[0] * cp[0] + ab[1] * cp[1] + ab[2] * cp[2];
    T d6 = ac[0] * cp[0] + ac[1] * cp[1] + ac[2] * cp[2];
    const T one(1), zero(0);
    if (d1 <= zero && d2 <= zero) { bary[0] = one; bary[1] = zero; bary[2] = zero; *region = 1; return; }
    if (d3 >= zero && d4 <= d3) { bary[0] = zero; bary[1] = one; bary[2] = zero; *region = 2; return; }
    T vc = d1 * d4 - d3 * d2;
    if (vc <= zero && d1 >= zero && d3 <= zero) {
        T v = d1 / (d1 - d3);
        bary[0] = one - v; bary[1] = v; bary[2] = zero; *region = 4; return;
    }
    if (d6 >= zero && d5 <= d6) { bary[0] = zero; bary[1] = zero; bary[2] = one; *region = 3; return; }
    T vb = d5 * d2 - d1 * d6;
    if (vb <= zero && d2 >= zero && d6 <= zero) {
        T w = d2 / (d2 - d6);
        bary[0] = one - w; bary[1] = zero; bary[2] = w; *region = 6; return;
    }
    T va = d3 * d6 - d5 * d4;
    if (va <= zero && (d4 - d3) >= zero && (d5 - d6) >= zero) {
        T w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[0] = zero; bary[1] = one - w; bary[2] = w; *region = 5; return;
    }
    T den = one / (va + vb + vc);
    T v = vb * den, w = vc * den;
    bary[0] = one - v - w; bary[1] = v; bary[2] = w; *region = 0;
}

MPM_HD float tri_dist2(const MeshTri& t, const float p[3], float bary[3], int* region) {
    closest_on_triangle<float>(p, t.a, t.b, t.c, bary, region);
    float d2 = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float e = bary[0] * t.a[k] + bary[1] * t.b[k] + bary[2] * t.c[k] - p[k];
        d2 += e * e;
    }
    return d2;
}

// FP64 distance^2 to a triangle with each operation rounded on its own, in the order of the closest-point
// routine above, so near-ties between faces are decided the same way on every machine.
MPM_HD double tri_dist2_exact(const MeshTri& t, const double p[3], double bary[3], int* region) {
    double a[3], b[3], c[3], ab[3], ac[3], ap[3], bp[3], cp[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = t.a[k]; b[k] = t.b[k]; c[k] = t.c[k];
        ab[k] = dsub(b[k], a[k]); ac[k] = dsub(c[k], a[k]);
        ap[k] = dsub(p[k], a[k]); bp[k] = dsub(p[k], b[k]); cp[k] = dsub(p[k], c[k]);
    }
    auto dot = [](const double* u, const double* v) { return dadd(dadd(dmul(u[0], v[0]), dmul(u[1], v[1])), dmul(u[2], v[2])); };
    double d1 = dot(ab, ap), d2 = dot(ac, ap), d3 = dot(ab, bp), d4 = dot(ac, bp), d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d1 <= 0 && d2 <= 0) { bary[0] = 1; bary[1] = 0; bary[2] = 0; *region = 1; }
    else if (d3 >= 0 && d4 <= d3) { bary[0] = 0; bary[1] = 1; bary[2] = 0; *region = 2; }
    else {
        double vc = dsub(dmul(d1, d4), dmul(d3, d2));
        double vb = dsub(dmul(d5, d2), dmul(d1, d6));
        double va = dsub(dmul(d3, d6), dmul(d5, d4));
        if (vc <= 0 && d1 >= 0 && d3 <= 0) {
            double v = ddiv(d1, dsub(d1, d3));
            bary[0] = dsub(1.0, v); bary[1] = v; bary[2] = 0; *region = 4;
        } else if (d6 >= 0 && d5 <= d6) {
            bary[0] = 0; bary[1] = 0; bary[2] = 1; *region = 3;
        } else if (vb <= 0 && d2 >= 0 && d6 <= 0) {
            double w = ddiv(d2, dsub(d2, d6));
            bary[0] = dsub(1.0, w); bary[1] = 0; bary[2] = w; *region = 6;
        } else if (va <= 0 && dsub(d4, d3) >= 0 && dsub(d5, d6) >= 0) {
            double w = ddiv(dsub(d4, d3), dadd(dsub(d4, d3), dsub(d5, d6)));
            bary[0] = 0; bary[1] = dsub(1.0, w); bary[2] = w; *region = 5;
        } else {
            double den = ddiv(1.0, dadd(dadd(va, vb), vc));
            double v = dmul(vb, den), w = dmul(vc, den);
            bary[0] = dsub(dsub(1.0, v), w); bary[1] = v; bary[2] = w; *region = 0;
        }
    }
    double dd = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double q = dadd(dadd(dmul(bary[0], a[k]), dmul(bary[1], b[k])), dmul(bary[2], c[k]));
        double e = dsub(q, p[k]);
        dd = dadd(dd, dmul(e, e));
    }
    return dd;
}

struct MeshHit {
    int tri;    // index into the leaf-ordered triangle array, -1 when the mesh is empty
    float sign;
    float cp[3];  // closest point, local space
};

MPM_HD float box_dist2(const BvhNode& nd, const float p[3]) {
    float d = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float e = fmaxf(fmaxf(nd.lo[a] - p[a], p[a] - nd.hi[a]), 0.f);
        d += e * e;
    }
    return d;
}

// Running closest-triangle selection. Candidates whose FP32 distance is within `tol` (absolute, local
// units) of the best so far are compared again: if both give the same closest point (a shared edge or
// vertex) the result does not depend on the face and the lower face index is kept; otherwise the two are
// compared in FP64, ties going to the lower face index. Near the mesh's medial axis two faces can be
// equidistant to FP32 rounding, and the FP64 comparison picks the same face as an exact query would.
struct ClosestState {
    float best, lo2, hi2;
    double best_d;  // FP64 distance^2 of the best, once needed
    int region, face, tri;
    float bary[3], cp[3];

    MPM_HD void init() {
        best = lo2 = hi2 = 3.0e38f;
        best_d = -1.0;
        region = 0;
        face = 0x7fffffff;
        tri = -1;
    }

    MPM_HD void consider(const MeshTri* __restrict__ tris, int i, const float p[3], const double pd[3], float tol) {
        const MeshTri& t = tris[i];
        float b[3];
        int rg;
        float d2 = tri_dist2(t, p, b, &rg);
        if (d2 > hi2) return;
        float c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) c[k] = b[0] * t.a[k] + b[1] * t.b[k] + b[2] * t.c[k];
        update(tris, i, d2, b, rg, c, t.face, pd, tol);
    }

    // The state change for candidate i whose FP32 distance^2 d2, barycentrics b, region rg, closest point c
    // and face were already evaluated (consider() evaluates them first; the warp query evaluates 32 at once).
    MPM_HD void update(const MeshTri* __restrict__ tris, int i, float d2, const float b[3], int rg, const float c[3],
                       int tface, const double pd[3], float tol) {
        if (d2 > hi2) return;
        const MeshTri& t = tris[i];
        bool take;
        if (tri < 0 || d2 < lo2) {
            take = true;
            best_d = -1.0;
        } else {
            float sep = (c[0] - cp[0]) * (c[0] - cp[0]) + (c[1] - cp[1]) * (c[1] - cp[1]) + (c[2] - cp[2]) * (c[2] - cp[2]);
            if (sep <= tol * tol) {
                take = tface < face;
                if (take) best_d = -1.0;
            } else {
                double bd[3];
                int rd;
                if (best_d < 0.0) best_d = tri_dist2_exact(tris[tri], pd, bd, &rd);
                double cd = tri_dist2_exact(t, pd, bd, &rd);
                take = cd < best_d || (cd == best_d && tface < face);
                if (take) best_d = cd;
            }
        }
        if (take) {
            best = d2;
            float r = sqrtf(best);
            lo2 = fmaxf(r - tol, 0.f);
            lo2 *= lo2;
            hi2 = (r + tol) * (r + tol);
            region = rg;
            face = tface;
            tri = i;
#pragma unroll
            for (int k = 0; k < 3; ++k) { bary[k] = b[k]; cp[k] = c[k]; }
        }
    }

    // The FP32 pass above only chooses the face. The winner's closest point is evaluated again in FP64 (its
    // barycentrics and region by the exact-order routine, the point rounded to FP32 once from FP32-rounded
    // barycentrics u, v and 1 - u - v): near the surface the normal is (p - cp) / |p - cp|, and a closest
    // point carrying FP32 rounding would put an error of about ulp(p) / |p - cp| into it (4e-3 for a node
    // 2e-4 cells off the surface). The sign is the side of the feature's pseudonormal, in FP64.
    MPM_HD MeshHit finish(const MeshTri* __restrict__ tris, const float p[3], const double pd[3]) {
        MeshHit hit;
        hit.tri = tri;
        hit.sign = 1.f;
        if (tri < 0) return hit;
        const MeshTri& t = tris[tri];
        double bd[3];
        int rg;
        tri_dist2_exact(t, pd, bd, &rg);
        const double u = (float)bd[0], v = (float)bd[1], w = dsub(dsub(1.0, u), v);
        double cpd[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double a = t.a[k], b = t.b[k], c = t.c[k];
            cpd[k] = dadd(dadd(dmul(bd[0], a), dmul(bd[1], b)), dmul(bd[2], c));
            hit.cp[k] = (float)dadd(dadd(dmul(u, a), dmul(v, b)), dmul(w, c));
        }
        const float* pn = rg == 0 ? t.fn : (rg <= 3 ? t.vn[rg - 1] : t.en[rg - 4]);
        const double s = dadd(dadd(dmul(dsub(pd[0], cpd[0]), (double)pn[0]), dmul(dsub(pd[1], cpd[1]), (double)pn[1])),
                              dmul(dsub(pd[2], cpd[2]), (double)pn[2]));
        hit.sign = s >= 0.0 ? 1.f : -1.f;
        (void)p;
        return hit;
    }
};

// Closest triangle through the BVH (nearer child first, subtrees farther than the best pruned).
MPM_HD MeshHit mesh_closest(const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris, const float p[3],
                            float tol) {
    ClosestState st;
    st.init();
    const double pd[3] = {p[0], p[1], p[2]};
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode nd = nodes[stack[--sp]];
        if (box_dist2(nd, p) > st.hi2) continue;
        if (nd.count > 0) {
            for (int i = nd.start; i < nd.start + nd.count; ++i) st.consider(tris, i, p, pd, tol);
        } else if (sp < 62) {
            const BvhNode l = nodes[nd.start], r = nodes[nd.start + 1];
            float dl = box_dist2(l, p), dr = box_dist2(r, p);
            if (dl <= dr) { stack[sp++] = nd.start + 1; stack[sp++] = nd.start; }
            else { stack[sp++] = nd.start; stack[sp++] = nd.start + 1; }
        }
    }
    return st.finish(tris, p, pd);
}

// Leaf-ordered indices of the triangles within sqrt(R2) of c, in a fixed traversal order. Returns how many
// there are; writes at most max_out of them to out (out may be null).
MPM_HD int tris_within(const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris, const float c[3], float R2,
                       int32_t* out, int max_out) {
    int count = 0;
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode nd = nodes[stack[--sp]];
        if (box_dist2(nd, c) > R2) continue;
        if (nd.count > 0) {
            for (int i = nd.start; i < nd.start + nd.count; ++i) {
                float b[3];
                int rg;
                if (tri_dist2(tris[i], c, b, &rg) <= R2) {
                    if (out && count < max_out) out[count] = i;
                    ++count;
                }
            }
        } else if (sp < 62) {
            stack[sp++] = nd.start + 1;
            stack[sp++] = nd.start;
        }
    }
    return count;
}

// ---------------------------------------------------------------------------------------------------------
// Narrow-band voxel grid of a collider, in its local space over the bounding box grown by the margin.
// A voxel is FAR when every point in it is provably outside beyond the contact cutoff (or, for an open mesh,
// behind it beyond its thickness): collider_sdf's answer there cannot reach the band, so "far" is
// returned at once. Otherwise the voxel lists every triangle within d_c + 2r of its centre (d_c: the
// centre's distance to the mesh, r: the voxel's half diagonal), which contains the closest triangle and all
// ties of any point in the voxel, so the query over the list gives the same answer as over the whole mesh.
// Voxels whose list would exceed max_cand (deep inside a closed mesh) use the BVH.
// ---------------------------------------------------------------------------------------------------------
constexpr int kSdfFar = -1, kSdfUseBvh = -2;

MPM_HD void sdf_voxel_center(const SdfGridDev& s, int64_t v, float c[3], float* r) {
    const int i = (int)(v / ((int64_t)s.dims[1] * s.dims[2]));
    const int j = (int)((v / s.dims[2]) % s.dims[1]);
    const int k = (int)(v % s.dims[2]);
    c[0] = s.lo[0] + ((float)i + 0.5f) * s.h;
    c[1] = s.lo[1] + ((float)j + 0.5f) * s.h;
    c[2] = s.lo[2] + ((float)k + 0.5f) * s.h;
    *r = 0.8660254f * s.h * 1.0001f;  // half diagonal, rounded up
}

// Candidate count of voxel v, or kSdfFar / kSdfUseBvh; *R2 gets the candidate radius squared.
MPM_HD int sdf_voxel_classify(const ColliderDev& col, const BvhNode* __restrict__ nodes,
                              const MeshTri* __restrict__ tris, int64_t v, int max_cand, float* R2) {
    const SdfGridDev& s = col.sdf;
    float c[3], r;
    sdf_voxel_center(s, v, c, &r);
    const float tol = 1.0e-6f * (fmaxf(fmaxf(fabsf(c[0]), fabsf(c[1])), fabsf(c[2])) + col.mesh_scale);
    MeshHit h = mesh_closest(nodes, tris, c, tol);
    if (h.tri < 0) return kSdfFar;
    const float dc = sqrtf((c[0] - h.cp[0]) * (c[0] - h.cp[0]) + (c[1] - h.cp[1]) * (c[1] - h.cp[1]) +
                           (c[2] - h.cp[2]) * (c[2] - h.cp[2]));
    const float slack = 4.0f * tol + 1.0e-5f * (dc + r);
    if (dc - r > slack) {  // the voxel does not reach the surface: one sign for all its points
        if (h.sign > 0.f && dc - r > s.cutoff + slack) return kSdfFar;
        if (!col.closed && h.sign < 0.f && dc - r > s.thick + slack) return kSdfFar;
    }
    const float R = dc + 2.0f * r + slack;
    *R2 = R * R;
    const int n = tris_within(nodes, tris, c, *R2, nullptr, 0);
    return n > max_cand ? kSdfUseBvh : n;
}

// Closest triangle of a local point inside the collider's margin box; hit.tri == -2 for "far".
MPM_HD MeshHit mesh_closest_sdf(const ColliderDev& col, const BvhNode* __restrict__ nodes,
                                const MeshTri* __restrict__ tris, const int2* __restrict__ cells,
                                const int32_t* __restrict__ cand, const float p[3], float tol) {
    const SdfGridDev& s = col.sdf;
    if (!cells || !s.built) return mesh_closest(nodes, tris, p, tol);
    int vi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int i = (int)floorf((p[a] - s.lo[a]) / s.h);
        vi[a] = i < 0 ? 0 : (i >= s.dims[a] ? s.dims[a] - 1 : i);
    }
    const int2 cell = cells[s.cell_offset + ((int64_t)vi[0] * s.dims[1] + vi[1]) * s.dims[2] + vi[2]];
    if (cell.y == kSdfFar) {
        MeshHit far;
        far.tri = -2;
        far.sign = 1.f;
        return far;
    }
    if (cell.y == kSdfUseBvh) return mesh_closest(nodes, tris, p, tol);
    ClosestState st;
    st.init();
    const double pd[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < cell.y; ++i) st.consider(tris, cand[cell.x + i], p, pd, tol);
    return st.finish(tris, p, pd);
}

#ifdef __CUDA_ARCH__
// mesh_closest_sdf for a query that all 32 lanes of a warp share (the same p, every lane calls it): the lanes
// evaluate the distances to 32 candidates of the voxel's list at once, then every lane runs the same
// sequential state update over them in list order, so the result is the one-lane query's, bit for bit, in
// about a thirtieth of the dependent loads. FAR voxels and the BVH fallback are as in the one-lane query.
__device__ __forceinline__ MeshHit mesh_closest_sdf_warp(const ColliderDev& col, const BvhNode* __restrict__ nodes,
                                                        const MeshTri* __restrict__ tris,
                                                        const int2* __restrict__ cells,
                                                        const int32_t* __restrict__ cand, const float p[3],
                                                        float tol) {
    const SdfGridDev& s = col.sdf;
    if (!cells || !s.built) return mesh_closest(nodes, tris, p, tol);
    int vi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int i = (int)floorf((p[a] - s.lo[a]) / s.h);
        vi[a] = i < 0 ? 0 : (i >= s.dims[a] ? s.dims[a] - 1 : i);
    }
    const int2 cell = cells[s.cell_offset + ((int64_t)vi[0] * s.dims[1] + vi[1]) * s.dims[2] + vi[2]];
    if (cell.y == kSdfFar) {
        MeshHit far;
        far.tri = -2;
        far.sign = 1.f;
        return far;
    }
    if (cell.y == kSdfUseBvh) return mesh_closest(nodes, tris, p, tol);
    ClosestState st;
    st.init();
    const double pd[3] = {p[0], p[1], p[2]};
    const int lane = threadIdx.x & 31;
    float carry = 3.0e38f;  // smallest FP32 distance^2 of the candidates before this chunk
    for (int base = 0; base < cell.y; base += 32) {
        int idx = -1, rg = 0, face = 0;
        float d2 = 3.0e38f, b[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
        if (base + lane < cell.y) {
            idx = cand[cell.x + base + lane];
            const MeshTri& t = tris[idx];
            d2 = tri_dist2(t, p, b, &rg);
#pragma unroll
            for (int k = 0; k < 3; ++k) c[k] = b[0] * t.a[k] + b[1] * t.b[k] + b[2] * t.c[k];
            face = t.face;
        }
        // Skip that cannot change the result: the state's best stays within tol (in distance) of the smallest
        // FP32 distance seen so far (a candidate is taken either below lo2, or in the tie window when it is
        // exactly closer or the same point), so hi2 stays below (sqrt(min so far) + 2 tol)^2 and a candidate
        // beyond that is rejected by update()'s first test. The bound used, 4 tol and a relative 1e-4, leaves
        // room for chains of ties. pm = min of the candidates up to this one (a prefix minimum).
        float pm = d2;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, pm, o);
            if (lane >= o) pm = fminf(pm, y);
        }
        float before = __shfl_up_sync(0xffffffffu, pm, 1);
        before = fminf(carry, lane == 0 ? 3.0e38f : before);
        const float lim = sqrtf(before) + 4.0f * tol;
        const bool maybe = base + lane < cell.y && (before >= 3.0e38f || d2 <= lim * lim * 1.0001f);
        unsigned int live = __ballot_sync(0xffffffffu, maybe);
        carry = fminf(carry, __shfl_sync(0xffffffffu, pm, 31));
        while (live) {  // the possibly-relevant candidates, in list order
            const int q = __ffs(live) - 1;
            live &= live - 1;
            const float dq = __shfl_sync(0xffffffffu, d2, q);
            const float bq[3] = {__shfl_sync(0xffffffffu, b[0], q), __shfl_sync(0xffffffffu, b[1], q),
                                 __shfl_sync(0xffffffffu, b[2], q)};
            const float cq[3] = {__shfl_sync(0xffffffffu, c[0], q), __shfl_sync(0xffffffffu, c[1], q),
                                 __shfl_sync(0xffffffffu, c[2], q)};
            st.update(tris, __shfl_sync(0xffffffffu, idx, q), dq, bq, __shfl_sync(0xffffffffu, rg, q), cq,
                      __shfl_sync(0xffffffffu, face, q), pd, tol);
        }
    }
    return st.finish(tris, p, pd);
}
#endif

// Absolute distance tolerance of the FP32 comparison at point p: a few FP32 ulps of the coordinates involved.
MPM_HD float query_tol(const ColliderDev& c, const float p[3]) {
    float m = fmaxf(fmaxf(fabsf(p[0]), fabsf(p[1])), fabsf(p[2]));
    return 1.0e-6f * (m + c.mesh_scale);
}

// World point -> collider local space, M^-1 p, rounded like the reference's transform_point.
MPM_HD void to_local(const ColliderPose& c, const float p[3], float pl[3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
        pl[r] = fadd(fadd(fadd(fmul(c.Minv[r][0], p[0]), fmul(c.Minv[r][1], p[1])), fmul(c.Minv[r][2], p[2])), c.Minv[r][3]);
}

// True when p is inside the collider's local bounding box grown by its margin, the only region where
// collider_sdf can return a finite distance (colliders.py:47-49).
MPM_HD bool in_margin_box(const ColliderDev& c, const ColliderPose& pose, const float p[3]) {
    if (c.n_tris == 0) return false;
    float pl[3];
    to_local(pose, p, pl);
    bool in = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) in &= !(pl[a] < c.aabb_lo[a] - c.margin || pl[a] > c.aabb_hi[a] + c.margin);
    return in;
}

// False when collider_sdf at p is sure to return "far" (phi = 1e30, no contact): outside the margin box, or
// in a voxel of the narrow band classified FAR. Lets the candidate lists hold only points that can touch.
MPM_HD bool collider_may_touch(const ColliderDev& c, const ColliderPose& pose, const int2* __restrict__ cells,
                               const float p[3]) {
    if (c.n_tris == 0) return false;
    float pl[3];
    to_local(pose, p, pl);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (pl[a] < c.aabb_lo[a] - c.margin || pl[a] > c.aabb_hi[a] + c.margin) return false;
    const SdfGridDev& s = c.sdf;
    if (!cells || !s.built) return true;
    int vi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int i = (int)floorf((pl[a] - s.lo[a]) / s.h);
        vi[a] = i < 0 ? 0 : (i >= s.dims[a] ? s.dims[a] - 1 : i);
    }
    return cells[s.cell_offset + ((int64_t)vi[0] * s.dims[1] + vi[1]) * s.dims[2] + vi[2]].y != kSdfFar;
}

// colliders.py:40-65 -> (outward normal, phi); phi = 1e30 when outside the margin box or behind an open mesh
// kWarp: the query is shared by a whole warp (all lanes pass the same p) and uses mesh_closest_sdf_warp.
template <bool kWarp = false>
MPM_HD void collider_sdf(const ColliderDev& c, const ColliderPose& pose, const BvhNode* __restrict__ nodes,
                         const MeshTri* __restrict__ tris, const int2* __restrict__ cells,
                         const int32_t* __restrict__ cand, const float p[3], float thickness, float n[3], float* phi) {
    n[0] = 0.f; n[1] = 0.f; n[2] = 1.f;
    *phi = 1.0e30f;
    if (c.n_tris == 0) return;
    float pl[3];
    to_local(pose, p, pl);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (pl[a] < c.aabb_lo[a] - c.margin || pl[a] > c.aabb_hi[a] + c.margin) return;
    MeshHit h;
#ifdef __CUDA_ARCH__
    if constexpr (kWarp)
        h = mesh_closest_sdf_warp(c, nodes + c.node_offset, tris + c.tri_offset, cells, cand, pl, query_tol(c, pl));
    else
#endif
        h = mesh_closest_sdf(c, nodes + c.node_offset, tris + c.tri_offset, cells, cand, pl, query_tol(c, pl));
    if (h.tri < 0) return;  // empty mesh, or a far voxel
    // the offset to the surface in world space, its length and direction, in the reference's order
    const float off[3] = {fsub(pl[0], h.cp[0]), fsub(pl[1], h.cp[1]), fsub(pl[2], h.cp[2])};
    float d[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) d[r] = fdot3(pose.M[r], off);
    const float dist = fsqrt(fdot3(d, d));
    if (dist > 1.0e-9f) {
        const float k = fdiv(h.sign, dist);
        n[0] = fmul(d[0], k); n[1] = fmul(d[1], k); n[2] = fmul(d[2], k);
    } else {  // on the surface: the face normal mapped by the inverse transpose
        const float* fn = tris[c.tri_offset + h.tri].fn;
        float tn[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            tn[r] = fadd(fadd(fmul(pose.Minv[0][r], fn[0]), fmul(pose.Minv[1][r], fn[1])), fmul(pose.Minv[2][r], fn[2]));
        const float l = fsqrt(fdot3(tn, tn));
        n[0] = l > 0.f ? fdiv(tn[0], l) : 0.f;
        n[1] = l > 0.f ? fdiv(tn[1], l) : 0.f;
        n[2] = l > 0.f ? fdiv(tn[2], l) : 0.f;
    }
    if (!c.closed && h.sign < 0.f && dist > thickness) return;
    *phi = fmul(h.sign, dist);
}

// colliders.py:68-74: velocity of the collider material point at p (central difference of the pose in s)
MPM_HD void collider_velocity(const ColliderPose& c, const float p[3], float out[3]) {
    float pl[3];
    to_local(c, p, pl);
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = fadd(fdot3(c.dM[r], pl), c.dM[r][3]);
}

}  // namespace mpm

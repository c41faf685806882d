/* CPU oracle of the reference MLS-MPM substep. TEST INFRASTRUCTURE ONLY (see mpm_oracle.h).
 *
 * Each function below cites the reference source it restates. Expressions keep the reference's operand
 * order; the build uses -ffp-contract=off so no fused multiply-adds change the rounding. Third-party
 * built-ins of the reference (Warp's svd3 and mesh queries) are restated from published methods:
 *   svd3: one-sided Jacobi (Hestenes) in float64, results rounded to REAL, with Warp's output convention
 *         (U, V proper rotations, singular values descending, sign of det(F) on the last one);
 *   mesh query: closest point on a triangle (Ericson, Real-Time Collision Detection 5.1.5) over a median
 *         split BVH, sign from the angle-weighted pseudonormal of the closest feature (Baerentzen & Aanaes).
 */
#include "mpm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORACLE_DOUBLE
#define RSQRT(x) sqrt(x)
#define REXP(x) exp(x)
#define RLOG(x) log(x)
#define RFLOOR(x) floor(x)
#else
#define RSQRT(x) sqrtf(x)
#define REXP(x) expf(x)
#define RLOG(x) logf(x)
#define RFLOOR(x) floorf(x)
#endif

#define NODE(d, i, j, k) ((((size_t)(i) * (size_t)(d)->dims[1] + (size_t)(j)) * (size_t)(d)->dims[2] + (size_t)(k)) * 4)

static inline REAL rmax(REAL a, REAL b) { return a > b ? a : b; }
static inline REAL rmin(REAL a, REAL b) { return a < b ? a : b; }
static inline REAL rclamp(REAL x, REAL lo, REAL hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* ---- small matrix helpers (row-major 3x3), operand order as in the reference expressions ---- */

static void mat_mul(const REAL *a, const REAL *b, REAL *out) {
    REAL t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] + a[i * 3 + 2] * b[2 * 3 + j];
    memcpy(out, t, sizeof t);
}

static void mat_mul_t(const REAL *a, const REAL *b, REAL *out) { /* a * transpose(b) */
    REAL t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3 + 0] * b[j * 3 + 0] + a[i * 3 + 1] * b[j * 3 + 1] + a[i * 3 + 2] * b[j * 3 + 2];
    memcpy(out, t, sizeof t);
}

static void mat_vec(const REAL *a, const REAL *v, REAL *out) {
    REAL t[3];
    for (int i = 0; i < 3; ++i) t[i] = a[i * 3 + 0] * v[0] + a[i * 3 + 1] * v[1] + a[i * 3 + 2] * v[2];
    memcpy(out, t, sizeof t);
}

static inline REAL dot3(const REAL *a, const REAL *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline REAL len3(const REAL *a) { return RSQRT(dot3(a, a)); }

/* ---- svd3 (Warp built-in called at kernels.py:35,57,252) ---- */

static double det3d(const double *m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static void svd3_f64(const double *A, double *U, double *s, double *V) {
    double B[9];
    memcpy(B, A, sizeof B);
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    static const int PQ[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 80; ++sweep) {
        int rotated = 0;
        for (int r = 0; r < 3; ++r) {
            int p = PQ[r][0], q = PQ[r][1];
            double al = 0, be = 0, ga = 0;
            for (int i = 0; i < 3; ++i) {
                al += B[i * 3 + p] * B[i * 3 + p];
                be += B[i * 3 + q] * B[i * 3 + q];
                ga += B[i * 3 + p] * B[i * 3 + q];
            }
            if (ga == 0.0 || fabs(ga) <= 1e-17 * sqrt(al * be)) continue;
            rotated = 1;
            double zeta = (be - al) / (2.0 * ga);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
            for (int i = 0; i < 3; ++i) {
                double bp = B[i * 3 + p], bq = B[i * 3 + q];
                B[i * 3 + p] = c * bp - sn * bq;
                B[i * 3 + q] = sn * bp + c * bq;
                double vp = V[i * 3 + p], vq = V[i * 3 + q];
                V[i * 3 + p] = c * vp - sn * vq;
                V[i * 3 + q] = sn * vp + c * vq;
            }
        }
        if (!rotated) break;
    }
    double nrm[3];
    for (int k = 0; k < 3; ++k) nrm[k] = sqrt(B[k] * B[k] + B[3 + k] * B[3 + k] + B[6 + k] * B[6 + k]);
    for (int a = 0; a < 2; ++a) /* sort columns by norm, descending */
        for (int b = 0; b < 2 - a; ++b)
            if (nrm[b] < nrm[b + 1]) {
                double t = nrm[b]; nrm[b] = nrm[b + 1]; nrm[b + 1] = t;
                for (int i = 0; i < 3; ++i) {
                    t = B[i * 3 + b]; B[i * 3 + b] = B[i * 3 + b + 1]; B[i * 3 + b + 1] = t;
                    t = V[i * 3 + b]; V[i * 3 + b] = V[i * 3 + b + 1]; V[i * 3 + b + 1] = t;
                }
            }
    if (det3d(V) < 0)
        for (int i = 0; i < 3; ++i) { V[i * 3 + 2] = -V[i * 3 + 2]; B[i * 3 + 2] = -B[i * 3 + 2]; }
    for (int k = 0; k < 3; ++k) {
        s[k] = nrm[k];
        for (int i = 0; i < 3; ++i) U[i * 3 + k] = nrm[k] > 0 ? B[i * 3 + k] / nrm[k] : 0.0;
    }
    if (nrm[0] == 0) {
        for (int i = 0; i < 9; ++i) U[i] = (i % 4 == 0) ? 1.0 : 0.0;
    } else {
        if (nrm[1] == 0) { /* complete u1 orthogonal to u0 */
            int ax = 0;
            for (int a = 1; a < 3; ++a) if (fabs(U[a * 3]) < fabs(U[ax * 3])) ax = a;
            double e[3] = {0, 0, 0}; e[ax] = 1.0;
            double d = U[ax * 3];
            double w[3], n = 0;
            for (int i = 0; i < 3; ++i) { w[i] = e[i] - d * U[i * 3]; n += w[i] * w[i]; }
            n = sqrt(n);
            for (int i = 0; i < 3; ++i) U[i * 3 + 1] = w[i] / n;
        }
        if (nrm[2] == 0) {
            U[0 * 3 + 2] = U[1 * 3 + 0] * U[2 * 3 + 1] - U[2 * 3 + 0] * U[1 * 3 + 1];
            U[1 * 3 + 2] = U[2 * 3 + 0] * U[0 * 3 + 1] - U[0 * 3 + 0] * U[2 * 3 + 1];
            U[2 * 3 + 2] = U[0 * 3 + 0] * U[1 * 3 + 1] - U[1 * 3 + 0] * U[0 * 3 + 1];
        }
    }
    if (det3d(U) < 0) {
        for (int i = 0; i < 3; ++i) U[i * 3 + 2] = -U[i * 3 + 2];
        s[2] = -s[2];
    }
}

void orc_svd3(const REAL *A, REAL *U, REAL *sig, REAL *V) {
    double a[9], u[9], s[3], v[9];
    for (int i = 0; i < 9; ++i) a[i] = (double)A[i];
    svd3_f64(a, u, s, v);
    for (int i = 0; i < 9; ++i) { U[i] = (REAL)u[i]; V[i] = (REAL)v[i]; }
    for (int i = 0; i < 3; ++i) sig[i] = (REAL)s[i];
}

/* ---- constitutive models: kernels.py:30-89 ---- */

static void fixed_corotated_tau(const REAL *F, REAL mu, REAL lam, REAL *tau) { /* kernels.py:30-38 */
    REAL U[9], sig[3], V[9], R[9], FR[9];
    orc_svd3(F, U, sig, V);
    mat_mul_t(U, V, R);
    REAL J = sig[0] * sig[1] * sig[2];
    REAL two_mu = (REAL)2.0 * mu;
    for (int i = 0; i < 9; ++i) FR[i] = two_mu * (F[i] - R[i]);
    mat_mul_t(FR, F, tau);
    REAL iso = lam * J * (J - (REAL)1.0);
    tau[0] += iso; tau[4] += iso; tau[8] += iso;
}

static void safe_log3(const REAL *s, REAL *e) { /* kernels.py:41-43 */
    for (int i = 0; i < 3; ++i) e[i] = RLOG(rmax(s[i], (REAL)1.0e-4));
}

static void hencky_tau(const REAL *F, REAL mu, REAL lam, REAL *tau) { /* kernels.py:51-60 */
    REAL U[9], sig[3], V[9], eps[3], d[3], Ud[9];
    orc_svd3(F, U, sig, V);
    safe_log3(sig, eps);
    REAL tr = eps[0] + eps[1] + eps[2];
    REAL two_mu = (REAL)2.0 * mu;
    for (int i = 0; i < 3; ++i) d[i] = two_mu * eps[i] + lam * tr;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Ud[i * 3 + j] = U[i * 3 + j] * d[j];
    mat_mul_t(Ud, U, tau);
}

static void project_von_mises(const REAL *sig, REAL mu, REAL yield_stress, REAL *out) { /* kernels.py:63-72 */
    REAL eps[3], dev[3];
    safe_log3(sig, eps);
    REAL tr = eps[0] + eps[1] + eps[2];
    REAL third = tr / (REAL)3.0;
    for (int i = 0; i < 3; ++i) dev[i] = eps[i] - third;
    REAL n = len3(dev);
    REAL limit = yield_stress / ((REAL)2.0 * mu);
    if (n > limit) {
        REAL f = limit / n;
        for (int i = 0; i < 3; ++i) out[i] = REXP(third + dev[i] * f);
        return;
    }
    memcpy(out, sig, 3 * sizeof(REAL));
}

static void project_drucker_prager(const REAL *sig, REAL mu, REAL lam, REAL alpha, REAL *out) { /* kernels.py:75-89 */
    REAL eps[3], dev[3];
    safe_log3(sig, eps);
    REAL tr = eps[0] + eps[1] + eps[2];
    if (tr >= (REAL)0.0) { out[0] = out[1] = out[2] = (REAL)1.0; return; }
    REAL third = tr / (REAL)3.0;
    for (int i = 0; i < 3; ++i) dev[i] = eps[i] - third;
    REAL n = len3(dev);
    if (n < (REAL)1.0e-10) { memcpy(out, sig, 3 * sizeof(REAL)); return; }
    REAL dgamma = n + ((REAL)3.0 * lam + (REAL)2.0 * mu) / ((REAL)2.0 * mu) * tr * alpha;
    if (dgamma <= (REAL)0.0) { memcpy(out, sig, 3 * sizeof(REAL)); return; }
    REAL f = dgamma / n;
    for (int i = 0; i < 3; ++i) out[i] = REXP(eps[i] - dev[i] * f);
}

/* ---- B-spline stencil: kernels.py:16-27 ---- */

static inline REAL bspline_w(REAL fx, int i) {
    if (i == 0) return (REAL)0.5 * ((REAL)1.5 - fx) * ((REAL)1.5 - fx);
    if (i == 1) return (REAL)0.75 - (fx - (REAL)1.0) * (fx - (REAL)1.0);
    return (REAL)0.5 * (fx - (REAL)0.5) * (fx - (REAL)0.5);
}

/* Returns 0 when the stencil would leave the padded grid (also for NaN / inf positions); such a particle
 * neither scatters nor gathers. The reference never meets this on valid input (positions are clamped). */
static int stencil(const OrcDomain *d, const REAL *xp_world, int base[3], REAL fx[3]) {
    int ok = 1;
    for (int a = 0; a < 3; ++a) {
        REAL xp = (xp_world[a] - (REAL)d->origin[a]) * (REAL)d->inv_dx;
        REAL b = RFLOOR(xp - (REAL)0.5);
        int in = b >= (REAL)0 && b <= (REAL)(d->dims[a] - 3);
        ok &= in;
        base[a] = in ? (int)b : 0;
        fx[a] = xp - b;
    }
    return ok;
}

/* ---- p2g: kernels.py:92-140 ---- */

void orc_p2g(const OrcDomain *d, const OrcMaterial *mats, int n, const REAL *x, const REAL *v, const REAL *C,
             const REAL *F, const REAL *Jp, const int32_t *mat, REAL dt, REAL *grid, int threads) {
    const REAL p_vol = (REAL)d->p_vol, inv_dx = (REAL)d->inv_dx, dx = (REAL)d->dx;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
    for (int p = 0; p < n; ++p) {
        const OrcMaterial *m = &mats[mat[p]];
        REAL mu = (REAL)m->mu, lam = (REAL)m->lam, tau[9];
        if (m->model == 1 || m->model == 2) {
            hencky_tau(&F[9 * p], mu, lam, tau);
        } else if (m->model == 3) {
            REAL h = rmin(REXP((REAL)m->hardening * ((REAL)1.0 - Jp[p])), (REAL)m->max_hardening);
            fixed_corotated_tau(&F[9 * p], mu * h, lam * h, tau);
        } else {
            fixed_corotated_tau(&F[9 * p], mu, lam, tau);
        }
        REAL pm = (REAL)m->density * p_vol; /* p_mass = density * p_vol in FP32, warp/solver.py:91,116 */
        REAL k_stress = -dt * p_vol * (REAL)4.0 * inv_dx * inv_dx;
        REAL affine[9];
        for (int i = 0; i < 9; ++i) affine[i] = k_stress * tau[i] + pm * C[9 * p + i];
        int base[3];
        REAL fx[3], w0[3] = {0}, w1[3] = {0}, w2[3] = {0}, mv[3];
        if (!stencil(d, &x[3 * p], base, fx)) continue;
        for (int a = 0; a < 3; ++a) mv[a] = pm * v[3 * p + a];
        for (int i = 0; i < 3; ++i) { w0[i] = bspline_w(fx[0], i); w1[i] = bspline_w(fx[1], i); w2[i] = bspline_w(fx[2], i); }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    REAL w = w0[i] * w1[j] * w2[k];
                    REAL dpos[3] = {((REAL)i - fx[0]) * dx, ((REAL)j - fx[1]) * dx, ((REAL)k - fx[2]) * dx};
                    REAL ad[3], val[4];
                    mat_vec(affine, dpos, ad);
                    for (int a = 0; a < 3; ++a) val[a] = w * (mv[a] + ad[a]);
                    val[3] = w * pm;
                    REAL *g = &grid[NODE(d, base[0] + i, base[1] + j, base[2] + k)];
                    for (int a = 0; a < 4; ++a) {
                        if (threads > 1) {
#pragma omp atomic
                            g[a] += val[a];
                        } else {
                            g[a] += val[a];
                        }
                    }
                }
    }
}

/* ---- grid_update: kernels.py:143-180 ---- */

static void wall_contact(REAL *vel, int axis, REAL friction) { /* kernels.py:143-152 */
    REAL vn = (REAL)fabs((double)vel[axis]);
    vel[axis] = (REAL)0.0;
    REAL vt_len = len3(vel);
    if (vt_len > (REAL)0.0) {
        REAL f = rmax((REAL)0.0, (REAL)1.0 - friction * vn / vt_len);
        for (int a = 0; a < 3; ++a) vel[a] = vel[a] * f;
    }
}

void orc_grid_update(const OrcDomain *d, REAL dt, REAL *grid, int threads) {
    const int nx = d->dims[0], ny = d->dims[1], nz = d->dims[2];
    const REAL fr = (REAL)d->wall_friction;
    REAL g[3] = {(REAL)d->gravity[0], (REAL)d->gravity[1], (REAL)d->gravity[2]};
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                REAL *node = &grid[NODE(d, i, j, k)];
                REAL m = node[3];
                if (m <= (REAL)0.0) continue;
                REAL vel[3];
                for (int a = 0; a < 3; ++a) vel[a] = node[a] / m + dt * g[a];
                int idx[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    if (d->lo_on[a] && idx[a] <= d->wall_lo_node[a] && vel[a] < (REAL)0.0) wall_contact(vel, a, fr);
                    if (d->hi_on[a] && idx[a] >= d->wall_hi_node[a] && vel[a] > (REAL)0.0) wall_contact(vel, a, fr);
                }
                for (int a = 0; a < 3; ++a) node[a] = vel[a];
            }
}

/* ---- g2p: kernels.py:183-263 ---- */

void orc_g2p(const OrcDomain *d, const OrcMaterial *mats, int n, REAL *x, REAL *v, REAL *C, REAL *F, REAL *Jp,
             const int32_t *mat, REAL dt, const REAL *grid, int threads) {
    const REAL inv_dx = (REAL)d->inv_dx, dx = (REAL)d->dx;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
    for (int p = 0; p < n; ++p) {
        int base[3];
        REAL fx[3], w0[3] = {0}, w1[3] = {0}, w2[3] = {0};
        int inside = stencil(d, &x[3 * p], base, fx);
        for (int i = 0; i < 3; ++i) { w0[i] = bspline_w(fx[0], i); w1[i] = bspline_w(fx[1], i); w2[i] = bspline_w(fx[2], i); }
        REAL nv[3] = {0, 0, 0}, nC[9] = {0};
        for (int i = 0; i < 3 * inside; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    REAL w = w0[i] * w1[j] * w2[k];
                    REAL dpos[3] = {((REAL)i - fx[0]) * dx, ((REAL)j - fx[1]) * dx, ((REAL)k - fx[2]) * dx};
                    const REAL *gv = &grid[NODE(d, base[0] + i, base[1] + j, base[2] + k)];
                    for (int a = 0; a < 3; ++a) nv[a] = nv[a] + w * gv[a];
                    REAL cw = (REAL)4.0 * inv_dx * inv_dx * w;
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) nC[r * 3 + c] = nC[r * 3 + c] + cw * (gv[r] * dpos[c]);
                }
        for (int a = 0; a < 3; ++a) v[3 * p + a] = nv[a];
        memcpy(&C[9 * p], nC, sizeof nC);

        REAL nx[3];
        for (int a = 0; a < 3; ++a) nx[a] = x[3 * p + a] + dt * nv[a];
        for (int a = 0; a < 3; ++a) {
            if (d->lo_on[a] && nx[a] < (REAL)d->wall_lo[a]) nx[a] = (REAL)d->wall_lo[a];
            if (d->hi_on[a] && nx[a] > (REAL)d->wall_hi[a]) nx[a] = (REAL)d->wall_hi[a];
        }
        if (isfinite(nx[0]) && isfinite(nx[1]) && isfinite(nx[2]))
            for (int a = 0; a < 3; ++a) nx[a] = rclamp(nx[a], (REAL)d->clamp_lo[a], (REAL)d->clamp_hi[a]);
        for (int a = 0; a < 3; ++a) x[3 * p + a] = nx[a];

        REAL G[9], Fn[9];
        for (int i = 0; i < 9; ++i) G[i] = ((i % 4 == 0) ? (REAL)1.0 : (REAL)0.0) + dt * nC[i];
        mat_mul(G, &F[9 * p], Fn);
        const OrcMaterial *m = &mats[mat[p]];
        if (m->model == 0) { memcpy(&F[9 * p], Fn, sizeof Fn); continue; }
        REAL U[9], sig[3], V[9], ns[3];
        orc_svd3(Fn, U, sig, V);
        if (m->model == 1) {
            project_von_mises(sig, (REAL)m->mu, (REAL)m->yield_stress, ns);
        } else if (m->model == 2) {
            project_drucker_prager(sig, (REAL)m->mu, (REAL)m->lam, (REAL)m->alpha, ns);
        } else {
            REAL lo = (REAL)1.0 - (REAL)m->crit_c, hi = (REAL)1.0 + (REAL)m->crit_s;
            for (int a = 0; a < 3; ++a) ns[a] = rclamp(sig[a], lo, hi);
            Jp[p] = Jp[p] * (sig[0] * sig[1] * sig[2]) / (ns[0] * ns[1] * ns[2]);
        }
        REAL Ud[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ud[i * 3 + j] = U[i * 3 + j] * ns[j];
        mat_mul_t(Ud, V, &F[9 * p]);
    }
}

REAL orc_max_speed(int n, const REAL *v) { /* kernels.py:266-269 (a NaN never wins the max) */
    REAL vmax = 0;
    for (int p = 0; p < n; ++p) {
        REAL s = len3(&v[3 * p]);
        if (s > vmax) vmax = s;
    }
    return vmax;
}

/* ---- occupancy: kernels.py:272-298 ---- */

void orc_scatter_volume(const OrcDomain *d, int n, const REAL *x, REAL *grid_vol) {
    const REAL p_vol = (REAL)d->p_vol;
    for (int p = 0; p < n; ++p) {
        int base[3];
        REAL fx[3];
        if (!stencil(d, &x[3 * p], base, fx)) continue;
        for (int i = 0; i < 3; ++i) {
            REAL wi = bspline_w(fx[0], i);
            for (int j = 0; j < 3; ++j) {
                REAL wj = bspline_w(fx[1], j);
                for (int k = 0; k < 3; ++k)
                    grid_vol[NODE(d, base[0] + i, base[1] + j, base[2] + k) / 4] += wi * wj * bspline_w(fx[2], k) * p_vol;
            }
        }
    }
}

void orc_query_fill(const OrcDomain *d, int m, const REAL *pts, const REAL *grid_vol, uint8_t *out) {
    const REAL cell_vol = (REAL)pow(d->dx, 3.0); /* dx**3 in float64, warp/solver.py:254 */
    for (int q = 0; q < m; ++q) {
        int idx[3], inside = 1;
        for (int a = 0; a < 3; ++a) {
            REAL g = (pts[3 * q + a] - (REAL)d->origin[a]) * (REAL)d->inv_dx;
            idx[a] = (int)copysign(floor(fabs((double)g) + 0.5), (double)g); /* round half away from zero */
            if (idx[a] < 0 || idx[a] >= d->dims[a]) inside = 0;
        }
        out[q] = inside && grid_vol[NODE(d, idx[0], idx[1], idx[2]) / 4] >= (REAL)0.5 * cell_vol;
    }
}

/* ---- meshes: closest point + pseudonormal sign (Warp mesh_query_point_sign_normal, colliders.py:50) ---- */

typedef struct BvhNode {
    double lo[3], hi[3];
    int left, right, start, count;
} BvhNode;

typedef struct OrcMesh {
    int nv, nt, n_nodes;
    double *P;   /* nv*3 */
    int *T;      /* nt*3 */
    double *fn;  /* nt*3 face unit normals */
    double *en;  /* nt*9 edge pseudonormals for edges ab, bc, ca */
    double *vn;  /* nv*3 vertex pseudonormals */
    BvhNode *nodes;
    int *order;  /* triangle ids in leaf order */
} OrcMesh;

typedef struct EdgeRef { int a, b, face, slot; } EdgeRef;

static int edge_cmp(const void *x, const void *y) {
    const EdgeRef *p = (const EdgeRef *)x, *q = (const EdgeRef *)y;
    if (p->a != q->a) return p->a < q->a ? -1 : 1;
    if (p->b != q->b) return p->b < q->b ? -1 : 1;
    return p->face - q->face;
}

static double *g_centroid_key;
static int g_axis;
static int centroid_cmp(const void *x, const void *y) {
    double a = g_centroid_key[*(const int *)x * 3 + g_axis], b = g_centroid_key[*(const int *)y * 3 + g_axis];
    if (a != b) return a < b ? -1 : 1;
    return *(const int *)x - *(const int *)y;
}

static int bvh_build(OrcMesh *m, double *cent, int start, int count) {
    int id = m->n_nodes++;
    BvhNode *nd = &m->nodes[id];
    for (int a = 0; a < 3; ++a) { nd->lo[a] = DBL_MAX; nd->hi[a] = -DBL_MAX; }
    double clo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, chi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = start; i < start + count; ++i) {
        int t = m->order[i];
        for (int c = 0; c < 3; ++c) {
            const double *p = &m->P[3 * m->T[3 * t + c]];
            for (int a = 0; a < 3; ++a) { if (p[a] < nd->lo[a]) nd->lo[a] = p[a]; if (p[a] > nd->hi[a]) nd->hi[a] = p[a]; }
        }
        for (int a = 0; a < 3; ++a) { double v = cent[3 * t + a]; if (v < clo[a]) clo[a] = v; if (v > chi[a]) chi[a] = v; }
    }
    nd->start = start; nd->count = count; nd->left = nd->right = -1;
    if (count <= 4) return id;
    int axis = 0;
    for (int a = 1; a < 3; ++a) if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    g_centroid_key = cent; g_axis = axis;
    qsort(&m->order[start], (size_t)count, sizeof(int), centroid_cmp);
    int half = count / 2;
    int l = bvh_build(m, cent, start, half);
    int r = bvh_build(m, cent, start + half, count - half);
    m->nodes[id].left = l; m->nodes[id].right = r; m->nodes[id].count = 0;
    return id;
}

void *orc_mesh_new(int n_verts, const float *verts, int n_tris, const int *tris) {
    OrcMesh *m = (OrcMesh *)calloc(1, sizeof(OrcMesh));
    m->nv = n_verts; m->nt = n_tris;
    m->P = (double *)malloc(sizeof(double) * 3 * (size_t)(n_verts > 0 ? n_verts : 1));
    m->T = (int *)malloc(sizeof(int) * 3 * (size_t)(n_tris > 0 ? n_tris : 1));
    for (int i = 0; i < 3 * n_verts; ++i) m->P[i] = (double)verts[i];
    memcpy(m->T, tris, sizeof(int) * 3 * (size_t)n_tris);
    m->fn = (double *)calloc(3 * (size_t)(n_tris + 1), sizeof(double));
    m->en = (double *)calloc(9 * (size_t)(n_tris + 1), sizeof(double));
    m->vn = (double *)calloc(3 * (size_t)(n_verts + 1), sizeof(double));
    for (int f = 0; f < n_tris; ++f) {
        const double *a = &m->P[3 * tris[3 * f]], *b = &m->P[3 * tris[3 * f + 1]], *c = &m->P[3 * tris[3 * f + 2]];
        double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (l < 1e-300) l = 1e-300;
        for (int a2 = 0; a2 < 3; ++a2) m->fn[3 * f + a2] = n[a2] / l;
    }
    /* edge pseudonormals: sum of the unit normals of all faces that share the undirected edge */
    EdgeRef *E = (EdgeRef *)malloc(sizeof(EdgeRef) * 3 * (size_t)(n_tris + 1));
    for (int f = 0; f < n_tris; ++f)
        for (int s = 0; s < 3; ++s) {
            int a = tris[3 * f + s], b = tris[3 * f + (s + 1) % 3];
            E[3 * f + s] = (EdgeRef){a < b ? a : b, a < b ? b : a, f, s};
        }
    qsort(E, 3 * (size_t)n_tris, sizeof(EdgeRef), edge_cmp);
    for (int i = 0; i < 3 * n_tris;) {
        int j = i;
        double sum[3] = {0, 0, 0};
        while (j < 3 * n_tris && E[j].a == E[i].a && E[j].b == E[i].b) {
            for (int a = 0; a < 3; ++a) sum[a] += m->fn[3 * E[j].face + a];
            ++j;
        }
        for (int k = i; k < j; ++k)
            for (int a = 0; a < 3; ++a) m->en[9 * E[k].face + 3 * E[k].slot + a] = sum[a];
        i = j;
    }
    free(E);
    for (int f = 0; f < n_tris; ++f)
        for (int c = 0; c < 3; ++c) {
            const double *v0 = &m->P[3 * tris[3 * f + c]], *v1 = &m->P[3 * tris[3 * f + (c + 1) % 3]],
                         *v2 = &m->P[3 * tris[3 * f + (c + 2) % 3]];
            double e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]}, e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
            double den = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]) * sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
            if (den < 1e-300) den = 1e-300;
            double ca = (e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]) / den;
            ca = ca < -1 ? -1 : (ca > 1 ? 1 : ca);
            double ang = acos(ca);
            for (int a = 0; a < 3; ++a) m->vn[3 * tris[3 * f + c] + a] += ang * m->fn[3 * f + a];
        }
    /* median-split BVH over triangle centroids */
    double *cent = (double *)malloc(sizeof(double) * 3 * (size_t)(n_tris + 1));
    m->order = (int *)malloc(sizeof(int) * (size_t)(n_tris + 1));
    for (int f = 0; f < n_tris; ++f) {
        m->order[f] = f;
        for (int a = 0; a < 3; ++a)
            cent[3 * f + a] = (m->P[3 * tris[3 * f] + a] + m->P[3 * tris[3 * f + 1] + a] + m->P[3 * tris[3 * f + 2] + a]) / 3.0;
    }
    m->nodes = (BvhNode *)malloc(sizeof(BvhNode) * 2 * (size_t)(n_tris + 1));
    m->n_nodes = 0;
    if (n_tris > 0) bvh_build(m, cent, 0, n_tris);
    free(cent);
    return m;
}

void orc_mesh_free(void *mesh) {
    OrcMesh *m = (OrcMesh *)mesh;
    if (!m) return;
    free(m->P); free(m->T); free(m->fn); free(m->en); free(m->vn); free(m->nodes); free(m->order); free(m);
}

/* Ericson 5.1.5; region: 0 face, 1..3 vertex a..c, 4 edge ab, 5 edge bc, 6 edge ca */
static void closest_on_triangle(const double *p, const double *a, const double *b, const double *c, double bary[3],
                                int *region) {
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    for (int i = 0; i < 3; ++i) { ab[i] = b[i] - a[i]; ac[i] = c[i] - a[i]; ap[i] = p[i] - a[i]; bp[i] = p[i] - b[i]; cp[i] = p[i] - c[i]; }
#define D3(u, v) ((u)[0] * (v)[0] + (u)[1] * (v)[1] + (u)[2] * (v)[2])
    double d1 = D3(ab, ap), d2 = D3(ac, ap), d3 = D3(ab, bp), d4 = D3(ac, bp), d5 = D3(ab, cp), d6 = D3(ac, cp);
#undef D3
    if (d1 <= 0 && d2 <= 0) { bary[0] = 1; bary[1] = 0; bary[2] = 0; *region = 1; return; }
    if (d3 >= 0 && d4 <= d3) { bary[0] = 0; bary[1] = 1; bary[2] = 0; *region = 2; return; }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { double v = d1 / (d1 - d3); bary[0] = 1 - v; bary[1] = v; bary[2] = 0; *region = 4; return; }
    if (d6 >= 0 && d5 <= d6) { bary[0] = 0; bary[1] = 0; bary[2] = 1; *region = 3; return; }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { double w = d2 / (d2 - d6); bary[0] = 1 - w; bary[1] = 0; bary[2] = w; *region = 6; return; }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[0] = 0; bary[1] = 1 - w; bary[2] = w; *region = 5; return;
    }
    double den = 1.0 / (va + vb + vc);
    double v = vb * den, w = vc * den;
    bary[0] = 1 - v - w; bary[1] = v; bary[2] = w; *region = 0;
}

int orc_mesh_query(const void *mesh, const double p[3], double *sign, double *u, double *v, double *dist2) {
    const OrcMesh *m = (const OrcMesh *)mesh;
    if (m->nt == 0) return -1;
    double best = DBL_MAX, best_bary[3] = {0, 0, 0}, best_cp[3] = {0, 0, 0};
    int best_face = -1, best_region = 0;
    int stack[128], sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BvhNode *nd = &m->nodes[stack[--sp]];
        double bd = 0;
        for (int a = 0; a < 3; ++a) {
            double e = p[a] < nd->lo[a] ? nd->lo[a] - p[a] : (p[a] > nd->hi[a] ? p[a] - nd->hi[a] : 0);
            bd += e * e;
        }
        if (bd > best) continue;
        if (nd->left < 0) {
            for (int i = nd->start; i < nd->start + nd->count; ++i) {
                int f = m->order[i];
                const double *a = &m->P[3 * m->T[3 * f]], *b = &m->P[3 * m->T[3 * f + 1]], *c = &m->P[3 * m->T[3 * f + 2]];
                double bary[3], cp[3];
                int region;
                closest_on_triangle(p, a, b, c, bary, &region);
                double d2 = 0;
                for (int k = 0; k < 3; ++k) {
                    cp[k] = bary[0] * a[k] + bary[1] * b[k] + bary[2] * c[k];
                    double e = cp[k] - p[k];
                    d2 += e * e;
                }
                if (d2 < best || (d2 == best && f < best_face)) {
                    best = d2; best_face = f; best_region = region;
                    memcpy(best_bary, bary, sizeof bary); memcpy(best_cp, cp, sizeof cp);
                }
            }
        } else {
            stack[sp++] = nd->right;
            stack[sp++] = nd->left;
        }
    }
    const double *pn;
    int f = best_face;
    if (best_region == 0) pn = &m->fn[3 * f];
    else if (best_region <= 3) pn = &m->vn[3 * m->T[3 * f + best_region - 1]];
    else pn = &m->en[9 * f + 3 * (best_region - 4)];
    double s = (p[0] - best_cp[0]) * pn[0] + (p[1] - best_cp[1]) * pn[1] + (p[2] - best_cp[2]) * pn[2];
    *sign = s >= 0.0 ? 1.0 : -1.0;
    *u = best_bary[0];
    *v = best_bary[1];
    *dist2 = best;
    return f;
}

/* ---- collider pose and SDF: colliders.py:20-74 ---- */

static void qmul(const double *a, const double *b, double *o) {
    double ax = a[0], ay = a[1], az = a[2], aw = a[3], bx = b[0], by = b[1], bz = b[2], bw = b[3];
    o[0] = aw * bx + ax * bw + ay * bz - az * by;
    o[1] = aw * by - ax * bz + ay * bw + az * bx;
    o[2] = aw * bz + ax * by - ay * bx + az * bw;
    o[3] = aw * bw - ax * bx - ay * by - az * bz;
}

/* quat_slerp as q0 (q0^-1 q1)^s, evaluated in float64 from the REAL inputs */
static void quat_slerp(const REAL *q0r, const REAL *q1r, REAL s, double *out) {
    double q0[4], q1[4], c[4], d[4];
    for (int i = 0; i < 4; ++i) { q0[i] = (double)q0r[i]; q1[i] = (double)q1r[i]; }
    c[0] = -q0[0]; c[1] = -q0[1]; c[2] = -q0[2]; c[3] = q0[3];
    qmul(c, q1, d);
    double w = d[3] < -1 ? -1 : (d[3] > 1 ? 1 : d[3]);
    double angle = 2.0 * acos(w);
    double an = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (an < 1e-12) { memcpy(out, q0, sizeof q0); return; }
    double h = 0.5 * (double)s * angle, sh = sin(h);
    double step[4] = {d[0] / an * sh, d[1] / an * sh, d[2] / an * sh, cos(h)};
    qmul(q0, step, out);
}

static void collider_matrix(const OrcCollider *c, REAL s, REAL *M) { /* colliders.py:30-37, M is 4x4 row-major */
    REAL q0[4], q1[4], R[9], S[9], A[9], t[3];
    for (int i = 0; i < 4; ++i) { q0[i] = (REAL)c->q0[i]; q1[i] = (REAL)c->q1[i]; }
    double q[4];
    quat_slerp(q0, q1, s, q);
    REAL qr[4] = {(REAL)q[0], (REAL)q[1], (REAL)q[2], (REAL)q[3]};
    double x = qr[0], y = qr[1], z = qr[2], w = qr[3];
    double Rd[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                    2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                    2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};
    for (int i = 0; i < 9; ++i) {
        R[i] = (REAL)Rd[i];
        REAL s0 = (REAL)c->S0[i], s1 = (REAL)c->S1[i];
        S[i] = s0 + s * (s1 - s0);
    }
    mat_mul(R, S, A);
    for (int a = 0; a < 3; ++a) { REAL t0 = (REAL)c->t0[a], t1 = (REAL)c->t1[a]; t[a] = t0 + s * (t1 - t0); }
    for (int r = 0; r < 3; ++r) {
        M[r * 4 + 0] = A[r * 3 + 0]; M[r * 4 + 1] = A[r * 3 + 1]; M[r * 4 + 2] = A[r * 3 + 2]; M[r * 4 + 3] = t[r];
    }
    M[12] = 0; M[13] = 0; M[14] = 0; M[15] = 1;
}

static void inverse44(const REAL *M, REAL *out) { /* float64 Gauss-Jordan, rounded to REAL */
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? (double)M[r * 4 + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r) if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
        if (piv != col) for (int c = 0; c < 8; ++c) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
        double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            double f = a[r][col];
            if (f != 0) for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[r * 4 + c] = (REAL)a[r][c + 4];
}

static void xform_point(const REAL *M, const REAL *p, REAL *o) {
    REAL t[3];
    for (int r = 0; r < 3; ++r) t[r] = M[r * 4 + 0] * p[0] + M[r * 4 + 1] * p[1] + M[r * 4 + 2] * p[2] + M[r * 4 + 3];
    memcpy(o, t, sizeof t);
}

static void xform_vector(const REAL *M, const REAL *p, REAL *o) {
    REAL t[3];
    for (int r = 0; r < 3; ++r) t[r] = M[r * 4 + 0] * p[0] + M[r * 4 + 1] * p[1] + M[r * 4 + 2] * p[2];
    memcpy(o, t, sizeof t);
}

/* colliders.py:40-65: out = (normal xyz, phi); phi = 1e30 when far */
static void collider_sdf(const OrcCollider *c, const REAL *M, const REAL *Minv, const REAL *p, REAL thickness,
                         REAL *out) {
    out[0] = 0; out[1] = 0; out[2] = 1; out[3] = (REAL)1.0e30;
    REAL pl[3];
    xform_point(Minv, p, pl);
    for (int a = 0; a < 3; ++a)
        if (pl[a] < (REAL)c->aabb_lo[a] - (REAL)c->margin || pl[a] > (REAL)c->aabb_hi[a] + (REAL)c->margin) return;
    double pd[3] = {pl[0], pl[1], pl[2]}, sign, u, v, d2;
    int f = orc_mesh_query(c->mesh, pd, &sign, &u, &v, &d2);
    if (f < 0) return;
    const OrcMesh *m = (const OrcMesh *)c->mesh;
    REAL ur = (REAL)u, vr = (REAL)v, cp[3], off[3], dvec[3], n[3];
    for (int a = 0; a < 3; ++a)
        cp[a] = (REAL)((double)ur * m->P[3 * m->T[3 * f] + a] + (double)vr * m->P[3 * m->T[3 * f + 1] + a] +
                       (1.0 - (double)ur - (double)vr) * m->P[3 * m->T[3 * f + 2] + a]);
    for (int a = 0; a < 3; ++a) off[a] = pl[a] - cp[a];
    xform_vector(M, off, dvec);
    REAL dist = len3(dvec);
    REAL sg = (REAL)sign;
    if (dist > (REAL)1.0e-9) {
        REAL k = sg / dist;
        for (int a = 0; a < 3; ++a) n[a] = dvec[a] * k;
    } else {
        REAL MinvT[16], nl[3], tn[3];
        for (int r = 0; r < 4; ++r) for (int cc = 0; cc < 4; ++cc) MinvT[r * 4 + cc] = Minv[cc * 4 + r];
        for (int a = 0; a < 3; ++a) nl[a] = (REAL)m->fn[3 * f + a];
        xform_vector(MinvT, nl, tn);
        REAL l = len3(tn);
        for (int a = 0; a < 3; ++a) n[a] = l > 0 ? tn[a] / l : 0;
    }
    REAL phi = sg * dist;
    if (!c->closed && sg < (REAL)0.0 && dist > thickness) return;
    out[0] = n[0]; out[1] = n[1]; out[2] = n[2]; out[3] = phi;
}

static void collider_velocity(const OrcCollider *c, const REAL *Minv, REAL s, const REAL *p, REAL inv_frame_dt,
                              REAL *out) { /* colliders.py:68-74 */
    REAL pl[3], Mp[16], Mm[16], dM[16];
    xform_point(Minv, p, pl);
    const REAL h = (REAL)1.0e-3;
    collider_matrix(c, s + h, Mp);
    collider_matrix(c, s - h, Mm);
    REAL k = inv_frame_dt / ((REAL)2.0 * h);
    for (int i = 0; i < 16; ++i) dM[i] = (Mp[i] - Mm[i]) * k;
    xform_point(dM, pl, out);
}

void orc_collider_pose(const OrcCollider *c, REAL s, REAL inv_frame_dt, REAL *M16, REAL *Minv16, REAL *dM16) {
    REAL Mp[16], Mm[16];
    collider_matrix(c, s, M16);
    inverse44(M16, Minv16);
    const REAL h = (REAL)1.0e-3;
    collider_matrix(c, s + h, Mp);
    collider_matrix(c, s - h, Mm);
    REAL k = inv_frame_dt / ((REAL)2.0 * h);
    for (int i = 0; i < 16; ++i) dM16[i] = (Mp[i] - Mm[i]) * k;
}

void orc_grid_colliders(const OrcDomain *d, int n_col, const OrcCollider *cols, REAL s, REAL inv_frame_dt,
                        REAL *grid, int threads) { /* colliders.py:77-117 */
    if (n_col <= 0) return;
    REAL (*M)[16] = malloc(sizeof(REAL[16]) * (size_t)n_col), (*Mi)[16] = malloc(sizeof(REAL[16]) * (size_t)n_col);
    for (int c = 0; c < n_col; ++c) { collider_matrix(&cols[c], s, M[c]); inverse44(M[c], Mi[c]); }
    const REAL dx = (REAL)d->dx, thickness = (REAL)d->thickness, band = (REAL)d->band;
    const int nx = d->dims[0], ny = d->dims[1], nz = d->dims[2];
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) if (threads > 1)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                REAL *node = &grid[NODE(d, i, j, k)];
                if (node[3] <= (REAL)0.0) continue;
                REAL pos[3] = {(REAL)d->origin[0] + (REAL)i * dx, (REAL)d->origin[1] + (REAL)j * dx,
                               (REAL)d->origin[2] + (REAL)k * dx};
                REAL vel[3] = {node[0], node[1], node[2]};
                for (int c = 0; c < n_col; ++c) {
                    REAL r[4];
                    collider_sdf(&cols[c], M[c], Mi[c], pos, thickness, r);
                    if (r[3] < band) {
                        REAL vcol[3], rel[3], rt[3];
                        collider_velocity(&cols[c], Mi[c], s, pos, inv_frame_dt, vcol);
                        for (int a = 0; a < 3; ++a) rel[a] = vel[a] - vcol[a];
                        REAL vn = dot3(rel, r);
                        if (vn < (REAL)0.0) {
                            for (int a = 0; a < 3; ++a) rt[a] = rel[a] - vn * r[a];
                            REAL rt_len = len3(rt);
                            if (rt_len > (REAL)0.0) {
                                REAL f = rmax((REAL)0.0, (REAL)1.0 - (REAL)cols[c].friction * (-vn) / rt_len);
                                for (int a = 0; a < 3; ++a) rt[a] = rt[a] * f;
                            }
                            if (r[3] < (REAL)0.0)
                                for (int a = 0; a < 3; ++a) vel[a] = vcol[a] + rt[a];
                            else
                                for (int a = 0; a < 3; ++a) vel[a] = vcol[a] + rt[a] + vn * r[a];
                        }
                    }
                }
                node[0] = vel[0]; node[1] = vel[1]; node[2] = vel[2];
            }
    free(M); free(Mi);
}

void orc_project_particles(const OrcDomain *d, int n_col, const OrcCollider *cols, REAL s, REAL inv_frame_dt,
                           int n, REAL *x, REAL *v, int threads) { /* colliders.py:120-148 */
    if (n_col <= 0) return;
    REAL (*M)[16] = malloc(sizeof(REAL[16]) * (size_t)n_col), (*Mi)[16] = malloc(sizeof(REAL[16]) * (size_t)n_col);
    for (int c = 0; c < n_col; ++c) { collider_matrix(&cols[c], s, M[c]); inverse44(M[c], Mi[c]); }
    const REAL thickness = (REAL)d->thickness;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64) if (threads > 1)
    for (int p = 0; p < n; ++p) {
        REAL pos[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]}, vel[3] = {v[3 * p], v[3 * p + 1], v[3 * p + 2]};
        for (int c = 0; c < n_col; ++c) {
            REAL r[4];
            collider_sdf(&cols[c], M[c], Mi[c], pos, thickness, r);
            if (r[3] < (REAL)0.0) {
                for (int a = 0; a < 3; ++a) pos[a] = pos[a] - r[3] * r[a];
                REAL vcol[3], rel[3];
                collider_velocity(&cols[c], Mi[c], s, pos, inv_frame_dt, vcol);
                for (int a = 0; a < 3; ++a) rel[a] = vel[a] - vcol[a];
                REAL vn = dot3(rel, r);
                if (vn < (REAL)0.0)
                    for (int a = 0; a < 3; ++a) vel[a] = vel[a] - vn * r[a];
            }
        }
        for (int a = 0; a < 3; ++a) { x[3 * p + a] = pos[a]; v[3 * p + a] = vel[a]; }
    }
    free(M); free(Mi);
}

void orc_substep(const OrcDomain *d, const OrcMaterial *mats, int n_col, const OrcCollider *cols, int n, REAL *x,
                 REAL *v, REAL *C, REAL *F, REAL *Jp, const int32_t *mat, REAL dt, REAL s, REAL inv_frame_dt,
                 REAL *grid, int threads) { /* warp/solver.py:187-211 */
    memset(grid, 0, sizeof(REAL) * 4 * (size_t)d->dims[0] * (size_t)d->dims[1] * (size_t)d->dims[2]);
    orc_p2g(d, mats, n, x, v, C, F, Jp, mat, dt, grid, threads);
    orc_grid_update(d, dt, grid, threads);
    orc_grid_colliders(d, n_col, cols, s, inv_frame_dt, grid, threads);
    orc_g2p(d, mats, n, x, v, C, F, Jp, mat, dt, grid, threads);
    orc_project_particles(d, n_col, cols, s, inv_frame_dt, n, x, v, threads);
}

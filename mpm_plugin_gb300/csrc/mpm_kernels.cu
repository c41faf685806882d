// sm_103a kernels of the MLS-MPM substep and of the particle-state bookkeeping around it.
//
// One substep = step_begin (substep fraction + collider poses, on the device) -> clear -> P2G -> grid update
// (normalise, gravity, walls, mesh colliders) -> G2P (+ particle projection out of colliders). Every kernel
// reads dt and s from a StepParams record in device memory, so a captured graph of one substep replays
// for every substep of an advance.
#include <cuda_runtime.h>

#include "mpm_device.cuh"
#include "mpm_internal.h"

namespace mpm {

// ------------------------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------------------------
__device__ __forceinline__ void red_add_v4(float4* addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

__device__ __forceinline__ void load_mat3(float* const* src, int64_t p, float M[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) M[i][j] = src[i * 3 + j][p];
}

__device__ __forceinline__ void store_mat3(float* const* dst, int64_t p, const float M[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) dst[i * 3 + j][p] = M[i][j];
}

// ------------------------------------------------------------------------------------------------------
// step_begin: advance the substep counter, set s = (k + 1) / steps (warp/solver.py:218-219) and the pose
// of every collider at s: slerped rotation times lerped stretch, lerped translation (colliders.py:30-37),
// its inverse, and d(pose)/dt by a central difference with h = 1e-3 (colliders.py:68-74).
// ------------------------------------------------------------------------------------------------------
// The pose is evaluated once per substep by one thread, with every operation rounded on its own (no fused
// multiply-adds): the collider velocity is a central difference with h = 1e-3, which magnifies last-bit
// differences of the pose about 500 times, so the pose follows the reference's operation order exactly.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

__device__ void qmul(const double* a, const double* b, double* o) {  // Hamilton product, (x, y, z, w)
    o[0] = dsub(dadd(dadd(dmul(a[3], b[0]), dmul(a[0], b[3])), dmul(a[1], b[2])), dmul(a[2], b[1]));
    o[1] = dadd(dadd(dsub(dmul(a[3], b[1]), dmul(a[0], b[2])), dmul(a[1], b[3])), dmul(a[2], b[0]));
    o[2] = dadd(dsub(dadd(dmul(a[3], b[2]), dmul(a[0], b[1])), dmul(a[1], b[0])), dmul(a[2], b[3]));
    o[3] = dsub(dsub(dsub(dmul(a[3], b[3]), dmul(a[0], b[0])), dmul(a[1], b[1])), dmul(a[2], b[2]));
}

__device__ void collider_matrix(const ColliderDev& c, float s, float M[3][4]) {
    // slerp q0 (q0^-1 q1)^s in float64 from the FP32 quaternions
    double q0[4], q1[4], cj[4], d[4];
    for (int i = 0; i < 4; ++i) { q0[i] = c.q0[i]; q1[i] = c.q1[i]; }
    cj[0] = -q0[0]; cj[1] = -q0[1]; cj[2] = -q0[2]; cj[3] = q0[3];
    qmul(cj, q1, d);
    double w = fmin(fmax(d[3], -1.0), 1.0);
    double angle = dmul(2.0, acos(w));
    double an = sqrt(dadd(dadd(dmul(d[0], d[0]), dmul(d[1], d[1])), dmul(d[2], d[2])));
    double q[4] = {q0[0], q0[1], q0[2], q0[3]};
    if (an >= 1e-12) {
        double h = dmul(dmul(0.5, (double)s), angle), sh = sin(h);
        double st[4] = {dmul(d[0] / an, sh), dmul(d[1] / an, sh), dmul(d[2] / an, sh), cos(h)};
        qmul(q0, st, q);
    }
    double x = (float)q[0], y = (float)q[1], z = (float)q[2], ww = (float)q[3];
    float R[3][3] = {
        {(float)dsub(1.0, dmul(2.0, dadd(dmul(y, y), dmul(z, z)))), (float)dmul(2.0, dsub(dmul(x, y), dmul(z, ww))),
         (float)dmul(2.0, dadd(dmul(x, z), dmul(y, ww)))},
        {(float)dmul(2.0, dadd(dmul(x, y), dmul(z, ww))), (float)dsub(1.0, dmul(2.0, dadd(dmul(x, x), dmul(z, z)))),
         (float)dmul(2.0, dsub(dmul(y, z), dmul(x, ww)))},
        {(float)dmul(2.0, dsub(dmul(x, z), dmul(y, ww))), (float)dmul(2.0, dadd(dmul(y, z), dmul(x, ww))),
         (float)dsub(1.0, dmul(2.0, dadd(dmul(x, x), dmul(y, y))))}};
    float S[3][3];
    for (int i = 0; i < 9; ++i) S[i / 3][i % 3] = fadd(c.S0[i], fmul(s, fsub(c.S1[i], c.S0[i])));
    for (int r = 0; r < 3; ++r) {
        for (int j = 0; j < 3; ++j) M[r][j] = fadd(fadd(fmul(R[r][0], S[0][j]), fmul(R[r][1], S[1][j])), fmul(R[r][2], S[2][j]));
        M[r][3] = fadd(c.t0[r], fmul(s, fsub(c.t1[r], c.t0[r])));
    }
}

__device__ void inverse_affine(const float M[3][4], float out[3][4]) {  // float64 elimination, rounded to FP32
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? (r < 3 ? (double)M[r][c] : (c == 3 ? 1.0 : 0.0)) : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; ++c) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
        double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] = dmul(a[col][c], inv);
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            double f = a[r][col];
            if (f != 0.0)
                for (int c = 0; c < 8; ++c) a[r][c] = dsub(a[r][c], dmul(f, a[col][c]));
        }
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) out[r][c] = (float)a[r][c + 4];
}

__global__ void k_step_begin(StepParams* sp, ColliderDev* cols, int n_col) {
    __shared__ float s_sh;
    if (threadIdx.x == 0) {
        StepParams p = *sp;
        if (p.steps > 0) {
            p.k += 1;
            p.s = (float)((double)(p.k + 1) / (double)p.steps);
            *sp = p;
        }
        s_sh = p.s;
    }
    __syncthreads();
    const float s = s_sh;
    const float inv_frame_dt = sp->inv_frame_dt;
    for (int c = threadIdx.x; c < n_col; c += blockDim.x) {
        ColliderDev& col = cols[c];
        float M[3][4], Mp[3][4], Mm[3][4], Mi[3][4];
        const float h = 1.0e-3f;
        collider_matrix(col, s, M);
        collider_matrix(col, fadd(s, h), Mp);
        collider_matrix(col, fsub(s, h), Mm);
        inverse_affine(M, Mi);
        float k = __fdiv_rn(inv_frame_dt, fmul(2.0f, h));
        for (int r = 0; r < 3; ++r)
            for (int j = 0; j < 4; ++j) {
                col.M[r][j] = M[r][j];
                col.Minv[r][j] = Mi[r][j];
                col.dM[r][j] = fmul(fsub(Mp[r][j], Mm[r][j]), k);
            }
    }
}

// ------------------------------------------------------------------------------------------------------
// P2G (kernels.py:92-140): stress by model, APIC affine momentum, scatter of (w (m v + A dpos), w m) to the
// 27 stencil nodes as one 16-byte vector reduction per node.
// ------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_p2g_scatter(Particles P, const Material* __restrict__ mats, GridDesc g,
                                                     const StepParams* __restrict__ sp, float4* __restrict__ grid,
                                                     unsigned int* fp64_lanes) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const float dt = sp->dt;
    const Material m = mats[P.mat[p]];
    float F[3][3], tau[3][3];
    load_mat3(P.F, p, F);
    if (m.model == 1 || m.model == 2) {
        hencky_tau(F, m.mu, m.lam, tau, fp64_lanes);
    } else if (m.model == 3) {
        float h = fminf(expf(m.hardening * (1.0f - P.Jp[p])), m.max_hardening);
        fixed_corotated_tau(F, m.mu * h, m.lam * h, tau, fp64_lanes);
    } else {
        fixed_corotated_tau(F, m.mu, m.lam, tau, fp64_lanes);
    }
    const float pm = m.p_mass;
    const float k_stress = -dt * g.p_vol * 4.0f * g.inv_dx * g.inv_dx;
    float A[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A[i][j] = k_stress * tau[i][j] + pm * P.C[i * 3 + j][p];
    int base[3];
    float fx[3], w[3][3], mv[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xp = (P.x[a][p] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx[a]);
        bspline_weights(fx[a], w[a]);
        mv[a] = pm * P.v[a][p];
    }
    if (!inside) return;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float wt = w[0][i] * w[1][j] * w[2][k];
                float dpos[3] = {((float)i - fx[0]) * g.dx, ((float)j - fx[1]) * g.dx, ((float)k - fx[2]) * g.dx};
                float val[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) val[a] = wt * (mv[a] + (A[a][0] * dpos[0] + A[a][1] * dpos[1] + A[a][2] * dpos[2]));
                red_add_v4(&grid[node_index(g, base[0] + i, base[1] + j, base[2] + k)], val[0], val[1], val[2], wt * pm);
            }
}

// ------------------------------------------------------------------------------------------------------
// Grid update (kernels.py:143-180) fused with mesh-collider contact (colliders.py:77-117).
// One CTA of 64 threads per 4x4x4 block; nodes without mass return at once.
// ------------------------------------------------------------------------------------------------------
__device__ __forceinline__ void wall_contact(float vel[3], int axis, float friction) {
    float vn = fabsf(vel[axis]);
    vel[axis] = 0.0f;
    float vt_len = sqrtf(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    if (vt_len > 0.0f) {
        float f = fmaxf(0.0f, 1.0f - friction * vn / vt_len);
        vel[0] *= f; vel[1] *= f; vel[2] *= f;
    }
}

__global__ void __launch_bounds__(64) k_grid_update(GridDesc g, float4* __restrict__ grid, const StepParams* __restrict__ sp,
                                                    const ColliderDev* __restrict__ cols, int n_col,
                                                    const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris) {
    const int64_t blk = blockIdx.x;
    const int l = threadIdx.x;
    const int bk = (int)(blk % g.nb[2]);
    const int bj = (int)((blk / g.nb[2]) % g.nb[1]);
    const int bi = (int)(blk / ((int64_t)g.nb[2] * g.nb[1]));
    const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
    float4* node = &grid[blk * 64 + l];
    float4 nv = *node;
    const float m = nv.w;
    if (!(m > 0.0f)) return;  // the reference skips m <= 0 (kernels.py:171-172)
    const float dt = sp->dt;
    float vel[3] = {nv.x / m + dt * g.gravity[0], nv.y / m + dt * g.gravity[1], nv.z / m + dt * g.gravity[2]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (g.lo_on[a] && idx[a] <= g.wall_lo_node[a] && vel[a] < 0.0f) wall_contact(vel, a, g.wall_friction);
        if (g.hi_on[a] && idx[a] >= g.wall_hi_node[a] && vel[a] > 0.0f) wall_contact(vel, a, g.wall_friction);
    }
    if (n_col > 0) {
        const float pos[3] = {g.origin[0] + (float)idx[0] * g.dx, g.origin[1] + (float)idx[1] * g.dx,
                              g.origin[2] + (float)idx[2] * g.dx};
        for (int c = 0; c < n_col; ++c) {
            const ColliderDev& col = cols[c];
            float n[3], phi;
            collider_sdf(col, nodes, tris, pos, g.thickness, n, &phi);
            if (phi < g.band) {
                float vcol[3];
                collider_velocity(col, pos, vcol);
                float rel[3] = {vel[0] - vcol[0], vel[1] - vcol[1], vel[2] - vcol[2]};
                float vn = rel[0] * n[0] + rel[1] * n[1] + rel[2] * n[2];
                if (vn < 0.0f) {
                    float rt[3] = {rel[0] - vn * n[0], rel[1] - vn * n[1], rel[2] - vn * n[2]};
                    float rt_len = sqrtf(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
                    if (rt_len > 0.0f) {
                        float f = fmaxf(0.0f, 1.0f - col.friction * (-vn) / rt_len);
                        rt[0] *= f; rt[1] *= f; rt[2] *= f;
                    }
                    if (phi < 0.0f) {  // behind the surface: no penetration
#pragma unroll
                        for (int a = 0; a < 3; ++a) vel[a] = vcol[a] + rt[a];
                    } else {  // in the band: friction only
#pragma unroll
                        for (int a = 0; a < 3; ++a) vel[a] = vcol[a] + rt[a] + vn * n[a];
                    }
                }
            }
        }
    }
    *node = make_float4(vel[0], vel[1], vel[2], m);
}

// ------------------------------------------------------------------------------------------------------
// G2P (kernels.py:183-263) fused with particle projection out of colliders (colliders.py:120-148).
// ------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_g2p(Particles P, const Material* __restrict__ mats, GridDesc g,
                                             const StepParams* __restrict__ sp, const float4* __restrict__ grid,
                                             const ColliderDev* __restrict__ cols, int n_col,
                                             const BvhNode* __restrict__ nodes, const MeshTri* __restrict__ tris,
                                             unsigned int* fp64_lanes) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const float dt = sp->dt;
    float xo[3];
    int base[3];
    float fx[3], w[3][3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        xo[a] = P.x[a][p];
        float xp = (xo[a] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx[a]);
        bspline_weights(fx[a], w[a]);
    }
    float nv[3] = {0.f, 0.f, 0.f}, nC[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    const float cscale = 4.0f * g.inv_dx * g.inv_dx;
    if (inside)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float wt = w[0][i] * w[1][j] * w[2][k];
                float dpos[3] = {((float)i - fx[0]) * g.dx, ((float)j - fx[1]) * g.dx, ((float)k - fx[2]) * g.dx};
                float4 gv = __ldg(&grid[node_index(g, base[0] + i, base[1] + j, base[2] + k)]);
                float gva[3] = {gv.x, gv.y, gv.z};
                float cw = cscale * wt;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    nv[a] += wt * gva[a];
#pragma unroll
                    for (int c = 0; c < 3; ++c) nC[a][c] += cw * (gva[a] * dpos[c]);
                }
            }
    float nx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        nx[a] = xo[a] + dt * nv[a];
        if (g.lo_on[a] && nx[a] < g.wall_lo[a]) nx[a] = g.wall_lo[a];
        if (g.hi_on[a] && nx[a] > g.wall_hi[a]) nx[a] = g.wall_hi[a];
    }
    // keep stencils inside the padded grid, but never turn a NaN into a finite position (kernels.py:236-240)
    if (isfinite(nx[0]) && isfinite(nx[1]) && isfinite(nx[2])) {
#pragma unroll
        for (int a = 0; a < 3; ++a) nx[a] = fminf(fmaxf(nx[a], g.clamp_lo[a]), g.clamp_hi[a]);
    }
    store_mat3(P.C, p, nC);

    float F[3][3], Fn[3][3];
    load_mat3(P.F, p, F);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            Fn[i][j] = ((i == 0 ? 1.0f : 0.0f) + dt * nC[i][0]) * F[0][j] + ((i == 1 ? 1.0f : 0.0f) + dt * nC[i][1]) * F[1][j] +
                       ((i == 2 ? 1.0f : 0.0f) + dt * nC[i][2]) * F[2][j];  // (I + dt C) F
    const Material m = mats[P.mat[p]];
    if (m.model != 0) {  // plastic models: SVD of the trial F and a return mapping on its singular values
        float U[3][3], sig[3], d[3], V[3][3], delta[3];
        svd3(Fn, U, sig, d, V, fp64_lanes);
        bool moved;
        if (m.model == 1) {
            moved = project_von_mises(sig, d, m.mu, m.yield_stress, delta);
        } else if (m.model == 2) {
            moved = project_drucker_prager(sig, d, m.mu, m.lam, m.alpha, delta);
        } else {
            float ratio;
            moved = project_snow(sig, d, m.clamp_lo, m.clamp_hi, delta, &ratio);
            P.Jp[p] = P.Jp[p] * ratio;
        }
        if (moved) {  // F = U diag(new) V^T, applied as F + U diag(new - old) V^T
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Fn[i][j] += U[i][0] * delta[0] * V[j][0] + U[i][1] * delta[1] * V[j][1] + U[i][2] * delta[2] * V[j][2];
        }
    }
    store_mat3(P.F, p, Fn);

    for (int c = 0; c < n_col; ++c) {  // push particles that ended up inside a collider onto its surface
        const ColliderDev& col = cols[c];
        float n[3], phi;
        collider_sdf(col, nodes, tris, nx, g.thickness, n, &phi);
        if (phi < 0.0f) {
#pragma unroll
            for (int a = 0; a < 3; ++a) nx[a] = nx[a] - phi * n[a];
            float vcol[3];
            collider_velocity(col, nx, vcol);
            float vn = (nv[0] - vcol[0]) * n[0] + (nv[1] - vcol[1]) * n[1] + (nv[2] - vcol[2]) * n[2];
            if (vn < 0.0f) {
#pragma unroll
                for (int a = 0; a < 3; ++a) nv[a] = nv[a] - vn * n[a];
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P.x[a][p] = nx[a];
        P.v[a][p] = nv[a];
    }
}

// ------------------------------------------------------------------------------------------------------
// max |v| (kernels.py:266-269); a NaN never wins, as in the oracle. Non-negative floats order like their bits.
// ------------------------------------------------------------------------------------------------------
__global__ void k_max_speed(Particles P, unsigned int* out) {
    float best = 0.0f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += (int64_t)gridDim.x * blockDim.x) {
        float vx = P.v[0][p], vy = P.v[1][p], vz = P.v[2][p];
        best = fmaxf(best, sqrtf(vx * vx + vy * vy + vz * vz));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(best));
}

// ------------------------------------------------------------------------------------------------------
// Particle-state I/O: host-order arrays (N,3) / (N,3,3) / (N,) <-> SoA, ordered by the insertion id.
// ------------------------------------------------------------------------------------------------------
__global__ void k_state_in(Particles P, int64_t off, int64_t n, const float* __restrict__ x, const float* __restrict__ v,
                           const float* __restrict__ C, const float* __restrict__ F, const float* __restrict__ Jp,
                           const int32_t* __restrict__ mat, const int32_t* __restrict__ emitter) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t p = off + i;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P.x[a][p] = x[i * 3 + a];
        P.v[a][p] = v[i * 3 + a];
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        P.C[e][p] = C ? C[i * 9 + e] : 0.0f;
        P.F[e][p] = F ? F[i * 9 + e] : ((e % 4 == 0) ? 1.0f : 0.0f);
    }
    P.Jp[p] = Jp ? Jp[i] : 1.0f;
    P.mat[p] = mat[i];
    P.emitter[p] = emitter[i];
    P.id[p] = (int32_t)p;
}

__global__ void k_state_out(Particles P, float* __restrict__ x, float* __restrict__ v, float* __restrict__ C,
                            float* __restrict__ F, float* __restrict__ Jp, int32_t* __restrict__ mat,
                            int32_t* __restrict__ emitter) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int64_t d = P.id[p];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (x) x[d * 3 + a] = P.x[a][p];
        if (v) v[d * 3 + a] = P.v[a][p];
    }
    if (C)
#pragma unroll
        for (int e = 0; e < 9; ++e) C[d * 9 + e] = P.C[e][p];
    if (F)
#pragma unroll
        for (int e = 0; e < 9; ++e) F[d * 9 + e] = P.F[e][p];
    if (Jp) Jp[d] = P.Jp[p];
    if (mat) mat[d] = P.mat[p];
    if (emitter) emitter[d] = P.emitter[p];
}

// ------------------------------------------------------------------------------------------------------
// Removal of particles more than one cell past an open side (warp/solver.py:222-240), order preserved.
// ------------------------------------------------------------------------------------------------------
__global__ void k_flag_escaped(Particles P, EscapeBounds eb, int32_t* __restrict__ keep_phys,
                               int32_t* __restrict__ keep_by_id, unsigned int* __restrict__ removed_per_mat) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xa = P.x[a][p];
        if (eb.open_lo[a] && xa < eb.lo[a]) out = true;
        if (eb.open_hi[a] && xa > eb.hi[a]) out = true;
    }
    keep_phys[p] = out ? 0 : 1;
    keep_by_id[P.id[p]] = out ? 0 : 1;
    if (out) atomicAdd(&removed_per_mat[P.mat[p]], 1u);
}

__global__ void k_compact(Particles src, Particles dst, const int32_t* __restrict__ keep_phys,
                          const int32_t* __restrict__ dst_index, const int32_t* __restrict__ new_id) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= src.n || !keep_phys[p]) return;
    int64_t q = dst_index[p];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dst.x[a][q] = src.x[a][p];
        dst.v[a][q] = src.v[a][p];
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        dst.C[e][q] = src.C[e][p];
        dst.F[e][q] = src.F[e][p];
    }
    dst.Jp[q] = src.Jp[p];
    dst.mat[q] = src.mat[p];
    dst.emitter[q] = src.emitter[p];
    dst.id[q] = new_id[src.id[p]];
}

// exclusive scan of int32 in three passes: per-CTA sums, one CTA over the sums, per-CTA scan + offset
constexpr int kScanTile = 1024;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh_warp, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? sh_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh_warp[lane] = s;
    }
    __syncthreads();
    int incl = x + (wid > 0 ? sh_warp[wid - 1] : 0);
    if (total) *total = sh_warp[(blockDim.x >> 5) - 1];
    return incl - v;
}

__global__ void k_scan_tiles(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ tile_sums) {
    __shared__ int sh[32];
    int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int total;
    block_exclusive_scan(v, sh, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t* __restrict__ sums, int64_t m, int32_t* __restrict__ grand_total) {
    __shared__ int sh[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < m; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        int v = i < m ? sums[i] : 0;
        int total;
        int ex = block_exclusive_scan(v, sh, &total);
        if (i < m) sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void k_scan_apply(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ tile_offsets,
                             int32_t* __restrict__ out) {
    __shared__ int sh[32];
    int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int ex = block_exclusive_scan(v, sh, nullptr);
    if (i < n) out[i] = ex + tile_offsets[blockIdx.x];
}

// ------------------------------------------------------------------------------------------------------
// Occupancy (kernels.py:272-298): B-spline splat of particle volume, then a nearest-node test.
// ------------------------------------------------------------------------------------------------------
__global__ void k_scatter_volume(Particles P, GridDesc g, float* __restrict__ vol) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    int base[3];
    float fx, w[3][3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xp = (P.x[a][p] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx);
        bspline_weights(fx, w[a]);
    }
    if (!inside) return;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                atomicAdd(&vol[node_index(g, base[0] + i, base[1] + j, base[2] + k)], w[0][i] * w[1][j] * w[2][k] * g.p_vol);
}

__global__ void k_query_fill(GridDesc g, const float* __restrict__ vol, float cell_vol, int64_t m,
                             const float* __restrict__ pts, uint8_t* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int idx[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float gq = (pts[q * 3 + a] - g.origin[a]) * g.inv_dx;
        idx[a] = (int)copysignf(floorf(fabsf(gq) + 0.5f), gq);  // round half away from zero
        if (idx[a] < 0 || idx[a] >= g.dims[a]) inside = false;
    }
    out[q] = inside && vol[node_index(g, idx[0], idx[1], idx[2])] >= 0.5f * cell_vol ? 1 : 0;
}

// grid read-back: blocked layout -> C order (i, j, k) with 4 floats per node
__global__ void k_grid_unblock(GridDesc g, const float4* __restrict__ grid, float4* __restrict__ out) {
    int64_t n = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int k = (int)(q % g.dims[2]);
    int j = (int)((q / g.dims[2]) % g.dims[1]);
    int i = (int)(q / ((int64_t)g.dims[2] * g.dims[1]));
    out[q] = grid[node_index(g, i, j, k)];
}

// ------------------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------------------
static inline unsigned int blocks_for(int64_t n, int t) { return (unsigned int)((n + t - 1) / t); }

void launch_step_begin(cudaStream_t st, StepParams* sp, ColliderDev* cols, int n_col) {
    k_step_begin<<<1, 32, 0, st>>>(sp, cols, n_col);
}

void launch_p2g(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                float4* grid, unsigned int* fp64) {
    if (P.n == 0) return;
    k_p2g_scatter<<<blocks_for(P.n, 256), 256, 0, st>>>(P, mats, g, sp, grid, fp64);
}

void launch_grid_update(cudaStream_t st, const GridDesc& g, float4* grid, const StepParams* sp, const ColliderDev* cols,
                        int n_col, const BvhNode* nodes, const MeshTri* tris) {
    int64_t nblk = (int64_t)g.nb[0] * g.nb[1] * g.nb[2];
    k_grid_update<<<(unsigned int)nblk, 64, 0, st>>>(g, grid, sp, cols, n_col, nodes, tris);
}

void launch_g2p(cudaStream_t st, const Particles& P, const Material* mats, const GridDesc& g, const StepParams* sp,
                const float4* grid, const ColliderDev* cols, int n_col, const BvhNode* nodes, const MeshTri* tris,
                unsigned int* fp64) {
    if (P.n == 0) return;
    k_g2p<<<blocks_for(P.n, 256), 256, 0, st>>>(P, mats, g, sp, grid, cols, n_col, nodes, tris, fp64);
}

void launch_max_speed(cudaStream_t st, const Particles& P, unsigned int* out) {
    if (P.n == 0) return;
    unsigned int b = blocks_for(P.n, 256);
    if (b > 152 * 8) b = 152 * 8;
    k_max_speed<<<b, 256, 0, st>>>(P, out);
}

void launch_state_in(cudaStream_t st, const Particles& P, int64_t off, int64_t n, const float* x, const float* v,
                     const float* C, const float* F, const float* Jp, const int32_t* mat, const int32_t* emitter) {
    if (n == 0) return;
    k_state_in<<<blocks_for(n, 256), 256, 0, st>>>(P, off, n, x, v, C, F, Jp, mat, emitter);
}

void launch_state_out(cudaStream_t st, const Particles& P, float* x, float* v, float* C, float* F, float* Jp,
                      int32_t* mat, int32_t* emitter) {
    if (P.n == 0) return;
    k_state_out<<<blocks_for(P.n, 256), 256, 0, st>>>(P, x, v, C, F, Jp, mat, emitter);
}

void launch_flag_escaped(cudaStream_t st, const Particles& P, const EscapeBounds& eb, int32_t* keep_phys,
                         int32_t* keep_by_id, unsigned int* removed_per_mat) {
    if (P.n == 0) return;
    k_flag_escaped<<<blocks_for(P.n, 256), 256, 0, st>>>(P, eb, keep_phys, keep_by_id, removed_per_mat);
}

void launch_compact(cudaStream_t st, const Particles& src, const Particles& dst, const int32_t* keep_phys,
                    const int32_t* dst_index, const int32_t* new_id) {
    if (src.n == 0) return;
    k_compact<<<blocks_for(src.n, 256), 256, 0, st>>>(src, dst, keep_phys, dst_index, new_id);
}

int64_t scan_tile_count(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

void launch_exclusive_scan(cudaStream_t st, const int32_t* in, int64_t n, int32_t* out, int32_t* tile_tmp,
                           int32_t* total) {
    if (n == 0) return;
    int64_t tiles = scan_tile_count(n);
    k_scan_tiles<<<(unsigned int)tiles, kScanTile, 0, st>>>(in, n, tile_tmp);
    k_scan_sums<<<1, 1024, 0, st>>>(tile_tmp, tiles, total);
    k_scan_apply<<<(unsigned int)tiles, kScanTile, 0, st>>>(in, n, tile_tmp, out);
}

void launch_scatter_volume(cudaStream_t st, const Particles& P, const GridDesc& g, float* vol) {
    if (P.n == 0) return;
    k_scatter_volume<<<blocks_for(P.n, 256), 256, 0, st>>>(P, g, vol);
}

void launch_grid_unblock(cudaStream_t st, const GridDesc& g, const float4* grid, float4* out) {
    int64_t n = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
    k_grid_unblock<<<blocks_for(n, 256), 256, 0, st>>>(g, grid, out);
}

void launch_query_fill(cudaStream_t st, const GridDesc& g, const float* vol, float cell_vol, int64_t m,
                       const float* pts, uint8_t* out) {
    if (m == 0) return;
    k_query_fill<<<blocks_for(m, 256), 256, 0, st>>>(g, vol, cell_vol, m, pts, out);
}

}  // namespace mpm

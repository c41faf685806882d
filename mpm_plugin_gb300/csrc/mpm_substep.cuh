// One MLS-MPM substep, item by item: the collider pose of the substep, P2G of one particle, the grid update
// of one node, collider contact of one node or particle, and G2P of one particle. The kernels in
// mpm_substep_kernels.cuh call these per thread (or per warp for shared contact queries); the same
// functions compile for the host, so the CPU tests run exactly this code against the oracle.
#pragma once

#include "mpm_device.cuh"

namespace mpm {

// The pose is evaluated once per substep by one thread, with every operation rounded on its own (no fused
// multiply-adds): the collider velocity is a central difference with h = 1e-3, which magnifies last-bit
// differences of the pose about 500 times, so the pose follows the reference's operation order exactly.
MPM_HD void qmul(const double* a, const double* b, double* o) {  // Hamilton product, (x, y, z, w)
    o[0] = dsub(dadd(dadd(dmul(a[3], b[0]), dmul(a[0], b[3])), dmul(a[1], b[2])), dmul(a[2], b[1]));
    o[1] = dadd(dadd(dsub(dmul(a[3], b[1]), dmul(a[0], b[2])), dmul(a[1], b[3])), dmul(a[2], b[0]));
    o[2] = dadd(dsub(dadd(dmul(a[3], b[2]), dmul(a[0], b[1])), dmul(a[1], b[0])), dmul(a[2], b[3]));
    o[3] = dsub(dsub(dsub(dmul(a[3], b[3]), dmul(a[0], b[0])), dmul(a[1], b[1])), dmul(a[2], b[2]));
}

MPM_HD void collider_matrix(const ColliderDev& c, float s, float M[3][4]) {
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

MPM_HD void inverse_affine(const float M[3][4], float out[3][4]) {  // float64 elimination, rounded to FP32
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


// Collider pose at substep fraction s: M, its inverse, and dM/dt by a central difference in s with
// h = 1e-3 scaled by 1 / frame_dt (colliders.py:30-37, 68-74).
MPM_HD void collider_pose_at(const ColliderDev& col, float s, float inv_frame_dt, ColliderPose& out) {
    float M[3][4], Mp[3][4], Mm[3][4], Mi[3][4];
    const float h = 1.0e-3f;
    collider_matrix(col, s, M);
    collider_matrix(col, fadd(s, h), Mp);
    collider_matrix(col, fsub(s, h), Mm);
    inverse_affine(M, Mi);
    float k = fdiv(inv_frame_dt, fmul(2.0f, h));
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 4; ++j) {
            out.M[r][j] = M[r][j];
            out.Minv[r][j] = Mi[r][j];
            out.dM[r][j] = fmul(fsub(Mp[r][j], Mm[r][j]), k);
        }
}

// ------------------------------------------------------------------------------------------------------
// P2G of one particle (kernels.py:92-140): stress by model, APIC affine momentum, scatter of
// (w (m v + A dpos), w m) to the 27 stencil nodes as one 16-byte vector reduction per node.
// ------------------------------------------------------------------------------------------------------
MPM_HD void grid_add(float4* addr, float a, float b, float c, float d) {
#ifdef __CUDA_ARCH__
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
#else
    addr->x += a; addr->y += b; addr->z += c; addr->w += d;
#endif
}

MPM_HD void load_mat3(float* const* src, int64_t p, float M[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) M[i][j] = src[i * 3 + j][p];
}

MPM_HD void store_mat3(float* const* dst, int64_t p, const float M[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) dst[i * 3 + j][p] = M[i][j];
}

// Asks for the line holding *addr in L1 without waiting for it (a hint: no register, no fault on any address).
MPM_HD void prefetch_l1(const void* addr) {
#ifdef __CUDA_ARCH__
    asm volatile("prefetch.global.L1 [%0];" ::"l"(addr));
#else
    (void)addr;
#endif
}

// Adds grid block b to the active list of this substep unless it is there already.
MPM_HD void mark_block(int64_t b, unsigned int* __restrict__ flags, int32_t* __restrict__ list,
                       unsigned int* __restrict__ count) {
#ifdef __CUDA_ARCH__
    if (flags[b] == 0u && atomicExch(&flags[b], 1u) == 0u) list[atomicAdd(count, 1u)] = (int32_t)b;
#else
    if (flags[b] == 0u) {
        flags[b] = 1u;
        list[(*count)++] = (int32_t)b;
    }
#endif
}

// Kirchhoff stress of one particle from the SVD of its deformation gradient, F = U diag(sig) V^T with
// d = sig - 1 (kernels.py:117-124): Hencky for von Mises and Drucker-Prager, fixed-corotated with snow
// hardening exp(xi (1 - Jp)) capped at max_hardening, plain fixed-corotated otherwise. Stored as the six
// entries xx, yy, zz, xy, xz, yz of the symmetric tensor.
MPM_HD void tau_from_svd(const Material& m, float jp, const float U[3][3], const float sig[3], const float d[3],
                         float tau6[6]) {
    float g[3], tau[3][3];
    if (m.model == 1 || m.model == 2) {
        hencky_principal(m.mu, m.lam, sig, d, g);
    } else if (m.model == 3) {
        float h = fminf(expf(m.hardening * (1.0f - jp)), m.max_hardening);
        corotated_principal(m.mu * h, m.lam * h, sig, d, g);
    } else {
        corotated_principal(m.mu, m.lam, sig, d, g);
    }
    sym_from_diag(U, g, tau);
    tau6[0] = tau[0][0];
    tau6[1] = tau[1][1];
    tau6[2] = tau[2][2];
    tau6[3] = tau[0][1];
    tau6[4] = tau[0][2];
    tau6[5] = tau[1][2];
}

// The stress of particle p from its stored F and Jp, for particles that enter the arena (added or loaded).
// Also stores the SVD's right basis V, from which the particle's next SVD starts (when the arena has it).
MPM_HD void particle_stress(const Particles& P, int64_t p, const Material* __restrict__ mats, unsigned int* fp64) {
    const Material m = mats[P.mat[p]];
    float F[3][3], U[3][3], sig[3], d[3], V[3][3], t[6];
    load_mat3(P.F, p, F);
    svd3(F, U, sig, d, V, fp64);
    tau_from_svd(m, P.Jp[p], U, sig, d, t);
#pragma unroll
    for (int e = 0; e < 6; ++e) P.tau[e][p] = t[e];
    if (P.Vq[0]) {
        float q[4];
        rotation_to_quat(V, q);
#pragma unroll
        for (int e = 0; e < 4; ++e) P.Vq[e][p] = q[e];
    }
}

// Node index of the stencil nodes base + (i, j, k): the blocked layout's index is a sum of one term per
// axis (node_index), so the 27 indices are x[i] + y[j] + z[k] from nine per-axis terms.
struct StencilIndex {
    int64_t x[3];
    int y[3], z[3];
    MPM_HD int64_t operator()(int i, int j, int k) const { return x[i] + (int64_t)(y[j] + z[k]); }
};

MPM_HD StencilIndex stencil_index(const GridDesc& g, const int base[3]) {
    StencilIndex s;
    const int64_t slab = (int64_t)g.nb[1] * g.nb[2] * 64;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int i = base[0] + d, j = base[1] + d, k = base[2] + d;
        s.x[d] = (int64_t)(i >> 2) * slab + (i & 3) * 16;
        s.y[d] = (j >> 2) * g.nb[2] * 64 + (j & 3) * 4;
        s.z[d] = (k >> 2) * 64 + (k & 3);
    }
    return s;
}

// Per-particle terms of P2G (kernels.py:93-140): stencil base and weights, p_mass v and the affine matrix
// A = -dt p_vol 4 inv_dx^2 tau + p_mass C. tau is the particle's stored Kirchhoff stress, computed from F at
// the end of the previous G2P (or when the particle entered), so P2G itself decomposes nothing. The
// contribution to stencil node (i, j, k) is w (p_mass v + A dpos) with dpos = ((i, j, k) - fx) dx; written as
// w (u0 + dA (i, j, k)) with dA = A dx and u0 = p_mass v - dA fx, the per-node work is a few multiply-adds by
// small integers along the stencil.
struct P2gTerms {
    int base[3];
    float w[3][3], u0[3], dA[3][3], pm;
};

// The fields P2G reads, straight from the particle arrays (GlobalFields) or from a CTA's staged copy.
struct GlobalFields {
    const Particles& P;
    int64_t p;
    MPM_HD float x(int a) const { return P.x[a][p]; }
    MPM_HD float v(int a) const { return P.v[a][p]; }
    MPM_HD float C(int e) const { return P.C[e][p]; }
    MPM_HD float tau(int e) const { return P.tau[e][p]; }
    MPM_HD int mat() const { return P.mat[p]; }
};

// A value this thread stored earlier in the same kernel, read again from L2 (so the compiler does not keep
// the stored value live in a register across the code in between).
MPM_HD float reload(const float* addr) {
#ifdef __CUDA_ARCH__
    return __ldcg(addr);
#else
    return *addr;
#endif
}

// The fields of a particle G2P has just written, for the scatter into the next substep's grid: x, v and C
// read back, the stress from the registers it was computed in.
struct ScatterFields {
    const Particles& P;
    int64_t p;
    const float* t;
    MPM_HD float x(int a) const { return reload(&P.x[a][p]); }
    MPM_HD float v(int a) const { return reload(&P.v[a][p]); }
    MPM_HD float C(int e) const { return reload(&P.C[e][p]); }
    MPM_HD float tau(int e) const { return t[e]; }
    MPM_HD int mat() const { return P.mat[p]; }
};

// False when the stencil leaves the grid (the particle scatters nothing).
template <class Fields>
MPM_HD bool p2g_terms_of(const Fields& f, const Material* __restrict__ mats, const GridDesc& g, float dt, P2gTerms& t) {
    const float t0 = f.tau(0), t1 = f.tau(1), t2 = f.tau(2), t3 = f.tau(3), t4 = f.tau(4), t5 = f.tau(5);
    const float tau[3][3] = {{t0, t3, t4}, {t3, t1, t5}, {t4, t5, t2}};
    t.pm = mats[f.mat()].p_mass;
    const float k_stress = -dt * g.p_vol * 4.0f * g.inv_dx * g.inv_dx;
    bool inside = true;
    float fx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float xp = (f.x(a) - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &t.base[a], &fx[a]);
        bspline_weights(fx[a], t.w[a]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) t.dA[i][j] = (k_stress * tau[i][j] + t.pm * f.C(i * 3 + j)) * g.dx;
        t.u0[i] = t.pm * f.v(i) - (t.dA[i][0] * fx[0] + t.dA[i][1] * fx[1] + t.dA[i][2] * fx[2]);
    }
    return inside;
}

MPM_HD bool p2g_terms(const Particles& P, int64_t p, const Material* __restrict__ mats, const GridDesc& g, float dt,
                      P2gTerms& t) {
    return p2g_terms_of(GlobalFields{P, p}, mats, g, dt, t);
}

// Momentum (x, y, z) and mass the particle adds to stencil node (i, j, k), i, j, k in 0..2. In unrolled
// loops the partial sums along i and j are common to the later nodes.
// On the device the x and y components go through the paired FP32 instructions (two fused multiply-adds
// or two products per instruction, each rounded as the scalar one): the same results in fewer instructions.
MPM_HD void p2g_node(const P2gTerms& t, int i, int j, int k, float out[4]) {
    const float wt = (t.w[0][i] * t.w[1][j]) * t.w[2][k];
#ifdef __CUDA_ARCH__
    float2 uxy = make_float2(t.u0[0], t.u0[1]);
    float uz = t.u0[2];
    if (i) {
        uxy = __ffma2_rn(make_float2(t.dA[0][0], t.dA[1][0]), make_float2((float)i, (float)i), uxy);
        uz = fmaf(t.dA[2][0], (float)i, uz);
    }
    if (j) {
        uxy = __ffma2_rn(make_float2(t.dA[0][1], t.dA[1][1]), make_float2((float)j, (float)j), uxy);
        uz = fmaf(t.dA[2][1], (float)j, uz);
    }
    if (k) {
        uxy = __ffma2_rn(make_float2(t.dA[0][2], t.dA[1][2]), make_float2((float)k, (float)k), uxy);
        uz = fmaf(t.dA[2][2], (float)k, uz);
    }
    const float2 w2 = make_float2(wt, wt);
    const float2 mxy = __fmul2_rn(w2, uxy), mzm = __fmul2_rn(w2, make_float2(uz, t.pm));
    out[0] = mxy.x;
    out[1] = mxy.y;
    out[2] = mzm.x;
    out[3] = mzm.y;
#else
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float u = t.u0[a];
        if (i) u = fmaf(t.dA[a][0], (float)i, u);
        if (j) u = fmaf(t.dA[a][1], (float)j, u);
        if (k) u = fmaf(t.dA[a][2], (float)k, u);
        out[a] = wt * u;
    }
    out[3] = wt * t.pm;
#endif
}

// Lists the grid blocks a stencil at `base` touches (one to eight 4x4x4 blocks). (Reading all eight flags
// first, as independent loads, made P2G 7 % slower on the mixed workload: measured.)
MPM_HD void mark_stencil_blocks(const GridDesc& g, const int base[3], unsigned int* flags, int32_t* list,
                                unsigned int* count) {
    const int b0[3] = {base[0] >> 2, base[1] >> 2, base[2] >> 2};
    const int b1[3] = {(base[0] + 2) >> 2, (base[1] + 2) >> 2, (base[2] + 2) >> 2};
    for (int bi = b0[0]; bi <= b1[0]; ++bi)
        for (int bj = b0[1]; bj <= b1[1]; ++bj)
            for (int bk = b0[2]; bk <= b1[2]; ++bk)
                mark_block(((int64_t)bi * g.nb[1] + bj) * g.nb[2] + bk, flags, list, count);
}

// Flags the grid blocks a stencil at `base` touches with plain stores (no list; k_list_blocks lists the
// flagged blocks after P2G). Lanes of the warp that would write the same flags leave it to the lowest of them.
MPM_HD void flag_stencil_blocks(const GridDesc& g, const int base[3], unsigned int* flags) {
    const int b0[3] = {base[0] >> 2, base[1] >> 2, base[2] >> 2};
    const int b1[3] = {(base[0] + 2) >> 2, (base[1] + 2) >> 2, (base[2] + 2) >> 2};
    const int64_t first = ((int64_t)b0[0] * g.nb[1] + b0[1]) * g.nb[2] + b0[2];
#ifdef __CUDA_ARCH__
    const unsigned long long key = (unsigned long long)first * 8u + (b1[0] - b0[0]) * 4u + (b1[1] - b0[1]) * 2u +
                                   (b1[2] - b0[2]);
    const unsigned int same = __match_any_sync(__activemask(), key);
    if ((threadIdx.x & 31u) != (unsigned int)(__ffs(same) - 1)) return;
#endif
    for (int bi = b0[0]; bi <= b1[0]; ++bi)
        for (int bj = b0[1]; bj <= b1[1]; ++bj)
            for (int bk = b0[2]; bk <= b1[2]; ++bk) flags[((int64_t)bi * g.nb[1] + bj) * g.nb[2] + bk] = 1u;
}

// P2G of one particle into `sink` (sink.begin(base) once, then sink.add(i, j, k, mv x, y, z, m) per node);
// false for a particle whose stencil leaves the padded grid (it scatters nothing).
template <class Sink>
MPM_HD bool p2g_particle_into(const Particles& P, int64_t p, const Material* __restrict__ mats, const GridDesc& g,
                              float dt, Sink& sink) {
    P2gTerms t;
    if (!p2g_terms(P, p, mats, g, dt, t)) return false;
    sink.begin(t.base);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float val[4];
                p2g_node(t, i, j, k, val);
                sink.add(t.base[0] + i, t.base[1] + j, t.base[2] + k, val[0], val[1], val[2], val[3]);
            }
    return true;
}

// Scatter straight into the global grid, optionally listing the grid blocks the stencil touches.
struct GlobalSink {
    const GridDesc* g;
    float4* grid;
    unsigned int* flags;
    int32_t* list;
    unsigned int* count;
    MPM_HD void begin(const int base[3]) {
        if (flags) mark_stencil_blocks(*g, base, flags, list, count);
    }
    MPM_HD void add(int i, int j, int k, float a, float b, float c, float d) {
        grid_add(&grid[node_index(*g, i, j, k)], a, b, c, d);
    }
};

// flags / list / count may be null (no active-block bookkeeping).
MPM_HD void p2g_particle(const Particles& P, int64_t p, const Material* __restrict__ mats, const GridDesc& g, float dt,
                         float4* __restrict__ grid, unsigned int* __restrict__ flags = nullptr,
                         int32_t* __restrict__ list = nullptr, unsigned int* __restrict__ count = nullptr) {
    GlobalSink sink{&g, grid, flags, list, count};
    p2g_particle_into(P, p, mats, g, dt, sink);
}

// ------------------------------------------------------------------------------------------------------
// Grid update of one node (kernels.py:143-180) fused with mesh-collider contact (colliders.py:77-117).
// ------------------------------------------------------------------------------------------------------
MPM_HD void wall_contact(float vel[3], int axis, float friction) {
    float vn = fabsf(vel[axis]);
    vel[axis] = 0.0f;
    float vt_len = sqrtf(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    if (vt_len > 0.0f) {
        float f = fmaxf(0.0f, 1.0f - friction * vn / vt_len);
        vel[0] *= f; vel[1] *= f; vel[2] *= f;
    }
}

// Normalise, gravity and wall contact of one node (kernels.py:155-180); false for a node without mass.
MPM_HD bool grid_node_walls(const GridDesc& g, float4* node, const int idx[3], float dt) {
    float4 nv = *node;
    const float m = nv.w;
    if (!(m > 0.0f)) return false;  // the reference skips m <= 0 (kernels.py:171-172)
    float vel[3] = {nv.x / m + dt * g.gravity[0], nv.y / m + dt * g.gravity[1], nv.z / m + dt * g.gravity[2]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (g.lo_on[a] && idx[a] <= g.wall_lo_node[a] && vel[a] < 0.0f) wall_contact(vel, a, g.wall_friction);
        if (g.hi_on[a] && idx[a] >= g.wall_hi_node[a] && vel[a] > 0.0f) wall_contact(vel, a, g.wall_friction);
    }
    *node = make_float4(vel[0], vel[1], vel[2], m);
    return true;
}

// World position of a grid node, rounded like the reference's origin + (i, j, k) * dx (colliders.py:101).
MPM_HD void node_position(const GridDesc& g, const int idx[3], float pos[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] = fadd(g.origin[a], fmul((float)idx[a], g.dx));
}

// True when some collider's query at pos can report contact (collider_may_touch).
MPM_HD bool near_any_collider(const float pos[3], const ColliderData& cd) {
    for (int c = 0; c < cd.n_col; ++c)
        if (collider_may_touch(cd.cols[c], cd.poses[c], cd.cells, pos)) return true;
    return false;
}

// True for the lane that stores a result: every thread, or lane 0 of a warp that works on one item together.
template <bool kWarp>
MPM_HD bool stores_result() {
#ifdef __CUDA_ARCH__
    return !kWarp || (threadIdx.x & 31) == 0;
#else
    return true;
#endif
}

// Mesh-collider contact of one node after the wall pass (colliders.py:77-117). kWarp: the whole warp works
// on this node (every lane passes the same node; the mesh queries are shared), lane 0 stores it.
template <bool kWarp = false>
MPM_HD void grid_node_colliders(const GridDesc& g, float4* node, const int idx[3], const ColliderData& cd) {
    float4 nv = *node;
    float vel[3] = {nv.x, nv.y, nv.z};
    float pos[3];
    node_position(g, idx, pos);
    for (int c = 0; c < cd.n_col; ++c) {
        const ColliderDev& col = cd.cols[c];
        float n[3], phi;
        collider_sdf<kWarp>(col, cd.poses[c], cd.nodes, cd.tris, cd.cells, cd.cand, pos, g.thickness, n, &phi);
        if (phi < g.band) {  // the response in the reference's operation order, each operation rounded
            float vcol[3];
            collider_velocity(cd.poses[c], pos, vcol);
            const float rel[3] = {fsub(vel[0], vcol[0]), fsub(vel[1], vcol[1]), fsub(vel[2], vcol[2])};
            const float vn = fdot3(rel, n);
            if (vn < 0.0f) {
                float rt[3] = {fsub(rel[0], fmul(vn, n[0])), fsub(rel[1], fmul(vn, n[1])), fsub(rel[2], fmul(vn, n[2]))};
                const float rt_len = fsqrt(fdot3(rt, rt));
                if (rt_len > 0.0f) {
                    const float f = fmaxf(0.0f, fsub(1.0f, fdiv(fmul(col.friction, -vn), rt_len)));
                    rt[0] = fmul(rt[0], f); rt[1] = fmul(rt[1], f); rt[2] = fmul(rt[2], f);
                }
                if (phi < 0.0f) {  // behind the surface: no penetration
#pragma unroll
                    for (int a = 0; a < 3; ++a) vel[a] = fadd(vcol[a], rt[a]);
                } else {  // in the band: friction only
#pragma unroll
                    for (int a = 0; a < 3; ++a) vel[a] = fadd(fadd(vcol[a], rt[a]), fmul(vn, n[a]));
                }
            }
        }
    }
    if (stores_result<kWarp>()) *node = make_float4(vel[0], vel[1], vel[2], nv.w);
}

// ------------------------------------------------------------------------------------------------------
// G2P of one particle (kernels.py:183-263) fused with projection out of colliders (colliders.py:120-148).
// ------------------------------------------------------------------------------------------------------
MPM_HD float4 load_node(const float4* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// FP64 redo of a Drucker-Prager or snow particle whose FP32 projection was active (the option to keep the
// return mapping at the clamp in double precision): the trial F rebuilt in FP64 from the stored F and the
// new C (both still in memory), then the SVD (eight double sweeps), the return mapping, the projected F, the
// snow hardening and the stress in FP64, rounded to FP32 only when stored.
// Only the G2P build for the option contains it, so the default build's registers never carry the FP64
// working set (an out-of-line call in the one build made the default G2P 28 % slower, measured).
MPM_HD void plastic_redo_fp64(const Particles& P, int64_t p, const Material& m, float dt, float jp_old,
                              float Fn_out[3][3], float* jp_out, float t_out[6]) {
    float F[3][3], C[3][3];
    load_mat3(P.F, p, F);
    load_mat3(P.C, p, C);
    double A[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            A[i][j] = ((i == 0 ? 1.0 : 0.0) + (double)dt * C[i][0]) * F[0][j] +
                      ((i == 1 ? 1.0 : 0.0) + (double)dt * C[i][1]) * F[1][j] +
                      ((i == 2 ? 1.0 : 0.0) + (double)dt * C[i][2]) * F[2][j];  // (I + dt C) F
    double U[3][3], sig[3], d[3], V[3][3], delta[3];
    svd3_dev_core<double, 8>(A, U, sig, d, V);
    double jp = jp_old;
    bool moved;
    if (m.model == 2) {
        moved = project_drucker_prager<double>(sig, d, m.mu, m.lam, m.alpha, delta);
    } else {
        double ratio;
        moved = project_snow<double>(sig, d, m.clamp_lo, m.clamp_hi, delta, &ratio);
        jp = jp * ratio;
    }
    if (moved) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                A[i][j] += U[i][0] * delta[0] * V[j][0] + U[i][1] * delta[1] * V[j][1] + U[i][2] * delta[2] * V[j][2];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            sig[i] += delta[i];
            d[i] += delta[i];
        }
    }
    double gp[3], tau[3][3];
    if (m.model == 2) {
        hencky_principal<double>(m.mu, m.lam, sig, d, gp);
    } else {
        const double h = min_t(exp_t((double)m.hardening * (1.0 - jp)), (double)m.max_hardening);
        corotated_principal<double>(m.mu * h, m.lam * h, sig, d, gp);
    }
    sym_from_diag<double>(U, gp, tau);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Fn_out[i][j] = (float)A[i][j];
    *jp_out = (float)jp;
    t_out[0] = (float)tau[0][0];
    t_out[1] = (float)tau[1][1];
    t_out[2] = (float)tau[2][2];
    t_out[3] = (float)tau[0][1];
    t_out[4] = (float)tau[0][2];
    t_out[5] = (float)tau[1][2];
}

// The inputs G2P reads (x, F, Jp, mat): from the particle arrays (ParticleIn), or from a copy a kernel has
// staged in shared memory (the tile G2P's planes). kPrefetch: request F's, Jp's and mat's lines ahead.
struct ParticleIn {
    static constexpr bool kPrefetch = true;
    const Particles& P;
    int64_t p;
    MPM_HD float x(int a) const { return P.x[a][p]; }
    MPM_HD float F(int e) const { return P.F[e][p]; }
    MPM_HD float Jp() const { return P.Jp[p]; }
    MPM_HD int mat() const { return P.mat[p]; }
};

// G2P of one particle gathering node velocities from `src` (src.stencil(base)(i, j, k) -> float4 of stencil
// node base + (i, j, k)); the new position goes to nx_out and, when tau_out is given, the stress stored for
// the next P2G to tau_out as well. kFp64Clamp builds in the FP64 redo at an active Drucker-Prager or snow
// clamp, taken where fp64_clamp is set. Inputs come from `in`, results are stored to particle p of P.
template <class Source, bool kFp64Clamp = false, class In = ParticleIn>
MPM_HD void g2p_particle_from(const Particles& P, int64_t p, const In& in, const Material* __restrict__ mats,
                              const GridDesc& g, float dt, const Source& src, unsigned int* fp64, float nx_out[3],
                              int fp64_clamp = 0, float* tau_out = nullptr, unsigned int* fp64_redo = nullptr) {
    // F, Jp and mat are read after the gather and the C store; their lines are requested now so that the
    // memory latency overlaps the gather
    if constexpr (In::kPrefetch) {
#pragma unroll
        for (int e = 0; e < 9; ++e) prefetch_l1(&P.F[e][p]);
        prefetch_l1(&P.Jp[p]);
        prefetch_l1(&P.mat[p]);
#pragma unroll
        for (int e = 0; e < 4; ++e) prefetch_l1(&P.Vq[e][p]);
    }
    float xo[3];
    int base[3];
    float fx[3], w[3][3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        xo[a] = in.x(a);
        float xp = (xo[a] - g.origin[a]) * g.inv_dx;
        inside &= stencil_axis(xp, g.dims[a], &base[a], &fx[a]);
        bspline_weights(fx[a], w[a]);
    }
    // v = sum w gv and C = 4 inv_dx^2 sum w gv (x) dpos (kernels.py:214-227). With dpos = ((i, j, k) - fx) dx,
    // sum w gv dpos_c = dx (S_c - fx_c v) where S_c = sum w gv idx_c; the sums are taken along k, then j, then
    // i, so each node costs six multiply-adds (w gv and idx_k w gv) instead of twenty-one.
    float nv[3] = {0.f, 0.f, 0.f}, S[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    if (inside) {
        const auto at = src.stencil(base);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float Q[3] = {0.f, 0.f, 0.f}, Qj[3] = {0.f, 0.f, 0.f}, Qk[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float R[3] = {0.f, 0.f, 0.f}, Rk[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float4 gv = at(i, j, k);
                    const float gva[3] = {gv.x, gv.y, gv.z};
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        R[a] = fmaf(w[2][k], gva[a], R[a]);
                        if (k) Rk[a] = fmaf((float)k * w[2][k], gva[a], Rk[a]);
                    }
                }
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    Q[a] = fmaf(w[1][j], R[a], Q[a]);
                    if (j) Qj[a] = fmaf((float)j * w[1][j], R[a], Qj[a]);
                    Qk[a] = fmaf(w[1][j], Rk[a], Qk[a]);
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                nv[a] = fmaf(w[0][i], Q[a], nv[a]);
                if (i) S[a][0] = fmaf((float)i * w[0][i], Q[a], S[a][0]);
                S[a][1] = fmaf(w[0][i], Qj[a], S[a][1]);
                S[a][2] = fmaf(w[0][i], Qk[a], S[a][2]);
            }
        }
    }
    const float cscale = 4.0f * g.inv_dx * g.inv_dx * g.dx;
    float nC[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) nC[a][c] = cscale * (S[a][c] - fx[c] * nv[a]);
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
    // x and v are final here: stored now, so their registers are free through the SVD
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P.x[a][p] = nx[a];
        P.v[a][p] = nv[a];
        nx_out[a] = nx[a];
    }

    float F[3][3], Fn[3][3];
#pragma unroll
    for (int e = 0; e < 9; ++e) F[e / 3][e % 3] = in.F(e);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            Fn[i][j] = ((i == 0 ? 1.0f : 0.0f) + dt * nC[i][0]) * F[0][j] + ((i == 1 ? 1.0f : 0.0f) + dt * nC[i][1]) * F[1][j] +
                       ((i == 2 ? 1.0f : 0.0f) + dt * nC[i][2]) * F[2][j];  // (I + dt C) F
    // SVD of the trial F: the plastic models project its singular values (kernels.py:241-262); all models then
    // take the next substep's stress from the same decomposition (F = U diag(sig + delta) V^T), which is what
    // P2G would get from decomposing the stored F again.
    const Material m = mats[in.mat()];
    float U[3][3], sig[3], d[3], V[3][3];
    {  // the SVD starts from the particle's previous right basis V0, and V is kept for the next substep
        float q[4], V0[3][3];
#pragma unroll
        for (int e = 0; e < 4; ++e) q[e] = P.Vq[e][p];
        quat_to_rotation(q, V0);
        svd3<kFp64Clamp>(Fn, U, sig, d, V, fp64, V0);  // the FP64 SVD fallback only in the FP64-clamp build
        rotation_to_quat(V, q);
#pragma unroll
        for (int e = 0; e < 4; ++e) P.Vq[e][p] = q[e];
    }
    const float jp_old = in.Jp();
    float jp = jp_old;
    bool redo = false;  // FP64 redo of a marginal Drucker-Prager or snow decision (or of every active clamp)
    if (m.model != 0) {
        float delta[3];
        bool moved, marginal = false;
        if (m.model == 1) {
            moved = project_von_mises(sig, d, m.mu, m.yield_stress, delta);
        } else if (m.model == 2) {
            moved = project_drucker_prager(sig, d, m.mu, m.lam, m.alpha, delta, kFp64Clamp ? &marginal : nullptr);
        } else {
            float ratio;
            moved = project_snow(sig, d, m.clamp_lo, m.clamp_hi, delta, &ratio, kFp64Clamp ? &marginal : nullptr);
            jp = jp * ratio;
        }
        // fp64_clamp 1: the lanes whose FP32 decision was marginal; 2: every lane whose clamp was active
        redo = kFp64Clamp && m.model >= 2 && (fp64_clamp == 2 ? moved : (fp64_clamp == 1 && marginal));
#ifdef __CUDA_ARCH__
        if (redo && fp64_redo) atomicAdd(fp64_redo, 1u);
#else
        if (redo && fp64_redo) *fp64_redo += 1u;
#endif
        if (moved) {  // F = U diag(new) V^T, applied as F + U diag(new - old) V^T
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Fn[i][j] += U[i][0] * delta[0] * V[j][0] + U[i][1] * delta[1] * V[j][1] + U[i][2] * delta[2] * V[j][2];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                sig[i] += delta[i];
                d[i] += delta[i];
            }
        }
    }
    float t[6];
    if constexpr (kFp64Clamp) {
        if (redo)
            plastic_redo_fp64(P, p, m, dt, jp_old, Fn, &jp, t);  // reads F and C before F is overwritten
        else
            tau_from_svd(m, jp, U, sig, d, t);
    } else {
        tau_from_svd(m, jp, U, sig, d, t);
    }
    store_mat3(P.F, p, Fn);
    if (m.model == 3) P.Jp[p] = jp;
#pragma unroll
    for (int e = 0; e < 6; ++e) {
        P.tau[e][p] = t[e];
        if (tau_out) tau_out[e] = t[e];
    }
}

// Grid nodes through the read-only data path (the grid is not written while a G2P kernel runs).
struct GlobalSource {
    const GridDesc* g;
    const float4* grid;
    struct Stencil {
        StencilIndex at;
        const float4* grid;
        MPM_HD float4 operator()(int i, int j, int k) const { return load_node(&grid[at(i, j, k)]); }
    };
    MPM_HD Stencil stencil(const int base[3]) const { return Stencil{stencil_index(*g, base), grid}; }
};

// Grid nodes from L2 (inside a kernel that also writes the grid in an earlier phase, where the read-only
// path could return lines of the previous substep).
struct CoherentSource {
    const GridDesc* g;
    const float4* grid;
    struct Stencil {
        StencilIndex at;
        const float4* grid;
        MPM_HD float4 operator()(int i, int j, int k) const {
#ifdef __CUDA_ARCH__
            return __ldcg(&grid[at(i, j, k)]);
#else
            return grid[at(i, j, k)];
#endif
        }
    };
    MPM_HD Stencil stencil(const int base[3]) const { return Stencil{stencil_index(*g, base), grid}; }
};

template <bool kFp64Clamp = false, class Source = GlobalSource>
MPM_HD void g2p_particle(const Particles& P, int64_t p, const Material* __restrict__ mats, const GridDesc& g, float dt,
                         const float4* grid, unsigned int* fp64, float nx_out[3], int fp64_clamp = 0,
                         float* tau_out = nullptr, unsigned int* fp64_redo = nullptr) {
    Source src{&g, grid};
    g2p_particle_from<Source, kFp64Clamp>(P, p, ParticleIn{P, p}, mats, g, dt, src, fp64, nx_out, fp64_clamp, tau_out,
                                          fp64_redo);
}

// Pushes a particle that ended up inside a collider onto its surface and removes its inward velocity
// relative to the collider (colliders.py:120-148). kWarp as for grid_node_colliders.
template <bool kWarp = false>
MPM_HD void project_particle(const Particles& P, int64_t p, const GridDesc& g, const ColliderData& cd) {
    float nx[3] = {P.x[0][p], P.x[1][p], P.x[2][p]}, nv[3] = {P.v[0][p], P.v[1][p], P.v[2][p]};
    for (int c = 0; c < cd.n_col; ++c) {
        const ColliderDev& col = cd.cols[c];
        float n[3], phi;
        collider_sdf<kWarp>(col, cd.poses[c], cd.nodes, cd.tris, cd.cells, cd.cand, nx, g.thickness, n, &phi);
        if (phi < 0.0f) {  // in the reference's operation order, each operation rounded
#pragma unroll
            for (int a = 0; a < 3; ++a) nx[a] = fsub(nx[a], fmul(phi, n[a]));
            float vcol[3];
            collider_velocity(cd.poses[c], nx, vcol);
            const float rel[3] = {fsub(nv[0], vcol[0]), fsub(nv[1], vcol[1]), fsub(nv[2], vcol[2])};
            const float vn = fdot3(rel, n);
            if (vn < 0.0f) {
#pragma unroll
                for (int a = 0; a < 3; ++a) nv[a] = fsub(nv[a], fmul(vn, n[a]));
            }
        }
    }
    if (!stores_result<kWarp>()) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P.x[a][p] = nx[a];
        P.v[a][p] = nv[a];
    }
}

}  // namespace mpm

// Host-side constants of a domain: the grid descriptor, the material table and the collider poses, in
// float64 as mpm_core/backends/warp/solver.py:37-71,154-172 computes them, rounded to FP32 for the kernels.
// Header-only and free of CUDA API calls, shared by the C-ABI and the CPU build used by the tests.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/mpm_gb300.h"
#include "mpm_types.h"

namespace mpm {

constexpr double kColliderThickness = 2.0;  // open-mesh colliders are solid this many cells deep, warp/solver.py:20

struct HostDomain {
    double dx, inv_dx, p_vol;
    double origin[3];
    int dims[3];
};

// A domain make_grid can build: a positive resolution and finite bounds with max > min on every axis
// (Domain.__post_init__, mpm_core/scene.py:44-51, refuses max <= min and resolutions below 4 on the Python
// side; a raw descriptor reaches this layer unchecked). Returns a message for the first violation, or nullptr.
inline const char* domain_problem(const MpmDomainDesc& dom) {
    if (dom.resolution <= 0) return "domain resolution must be positive";
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(dom.min[a]) || !std::isfinite(dom.max[a])) return "domain bounds must be finite";
        if (!(dom.max[a] > dom.min[a])) return "domain max must exceed min on every axis";
    }
    if (!std::isfinite(dom.wall_friction)) return "wall friction must be finite";
    return nullptr;
}

// mpm_core/scene.py:60-67 (dx, grid shape) and warp/solver.py:37-53 (padding, origin, walls, clamps)
inline GridDesc make_grid(const MpmDomainDesc& dom, const double gravity[3], int ppc, HostDomain* hd) {
    GridDesc g{};
    double size[3], longest = 0;
    for (int a = 0; a < 3; ++a) {
        size[a] = dom.max[a] - dom.min[a];
        longest = std::max(longest, size[a]);
    }
    hd->dx = longest / dom.resolution;
    hd->inv_dx = 1.0 / hd->dx;
    hd->p_vol = std::pow(hd->dx, 3.0) / ppc;
    for (int a = 0; a < 3; ++a) {
        int shape = std::max(1, (int)std::ceil(size[a] / hd->dx - 1e-6));
        hd->dims[a] = shape + 2 * kPad;
        hd->origin[a] = dom.min[a] - kPad * hd->dx;
        g.dims[a] = hd->dims[a];
        g.nb[a] = (hd->dims[a] + kBlock - 1) / kBlock;
        g.origin[a] = (float)hd->origin[a];
        g.gravity[a] = (float)gravity[a];
        g.lo_on[a] = dom.wall_lo[a] ? 1 : 0;
        g.hi_on[a] = dom.wall_hi[a] ? 1 : 0;
        g.wall_lo[a] = (float)dom.min[a];
        g.wall_hi[a] = (float)dom.max[a];
        g.clamp_lo[a] = (float)(hd->origin[a] + hd->dx);
        g.clamp_hi[a] = (float)(hd->origin[a] + (hd->dims[a] - 2) * hd->dx);
        // last node index at/below each lo wall and first at/above each hi wall, with a 1e-3 cell tolerance
        g.wall_lo_node[a] = (int)std::floor((dom.min[a] - hd->origin[a]) / hd->dx + 1e-3);
        g.wall_hi_node[a] = (int)std::ceil((dom.max[a] - hd->origin[a]) / hd->dx - 1e-3);
    }
    g.dx = (float)hd->dx;
    g.inv_dx = (float)hd->inv_dx;
    g.p_vol = (float)hd->p_vol;
    g.wall_friction = (float)dom.wall_friction;
    g.thickness = (float)(kColliderThickness * hd->dx);
    g.band = (float)hd->dx;
    return g;
}

// warp/solver.py:56-71 with MaterialParams.lame (materials.py:48-51) and the Drucker-Prager cone
// coefficient sqrt(2/3) 2 sin(phi) / (3 - sin(phi)) (warp/solver.py:263-265). *wave: P-wave speed with the
// worst-case snow hardening, for the CFL step (warp/solver.py:59-62).
inline Material make_material(const MpmMaterialDesc& d, double p_vol, double* wave) {
    double e = d.youngs_modulus, nu = d.poisson_ratio;
    double mu = e / (2 * (1 + nu)), lam = e * nu / ((1 + nu) * (1 - 2 * nu));
    double sphi = std::sin(d.friction_angle_deg * (M_PI / 180.0));
    double alpha = std::sqrt(2.0 / 3.0) * 2 * sphi / (3 - sphi);
    Material t{};
    t.model = d.model;
    t.mu = (float)mu;
    t.lam = (float)lam;
    t.yield_stress = (float)d.yield_stress;
    t.alpha = (float)alpha;
    t.hardening = (float)d.hardening;
    t.max_hardening = (float)d.max_hardening;
    t.clamp_lo = 1.0f - (float)d.critical_compression;
    t.clamp_hi = 1.0f + (float)d.critical_stretch;
    t.p_mass = (float)d.density * (float)p_vol;  // FP32 product, as numpy forms it (warp/solver.py:91)
    *wave = std::sqrt((lam + 2 * mu) * (d.model == MPM_MODEL_SNOW ? d.max_hardening : 1.0) / d.density);
    return t;
}

// ---- pose decomposition (mpm_core/geometry.py:30-50) ----

inline void svd3_host(const double A[9], double U[9], double s[3], double V[9]) {  // one-sided Jacobi, float64
    double B[9];
    std::memcpy(B, A, sizeof B);
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (auto& r : pq) {
            int p = r[0], q = r[1];
            double al = 0, be = 0, ga = 0;
            for (int i = 0; i < 3; ++i) {
                al += B[i * 3 + p] * B[i * 3 + p];
                be += B[i * 3 + q] * B[i * 3 + q];
                ga += B[i * 3 + p] * B[i * 3 + q];
            }
            if (ga == 0.0 || std::fabs(ga) <= 1e-17 * std::sqrt(al * be)) continue;
            rotated = true;
            double zeta = (be - al) / (2.0 * ga);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
            double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
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
    double n[3];
    for (int k = 0; k < 3; ++k) n[k] = std::sqrt(B[k] * B[k] + B[3 + k] * B[3 + k] + B[6 + k] * B[6 + k]);
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return n[a] > n[b]; });
    double B2[9], V2[9];
    for (int k = 0; k < 3; ++k) {
        s[k] = n[ord[k]];
        for (int i = 0; i < 3; ++i) {
            B2[i * 3 + k] = B[i * 3 + ord[k]];
            V2[i * 3 + k] = V[i * 3 + ord[k]];
        }
    }
    std::memcpy(V, V2, sizeof V2);
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) U[i * 3 + k] = s[k] > 0 ? B2[i * 3 + k] / s[k] : (i == k ? 1.0 : 0.0);
}

inline double det3(const double m[9]) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// World matrix -> translation, rotation quaternion (x, y, z, w), symmetric stretch; M = [R S | t].
inline void decompose(const float* m16, double t[3], double q[4], double S[9], double* min_sv) {
    double A[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A[r * 3 + c] = m16[r * 4 + c];
    for (int r = 0; r < 3; ++r) t[r] = m16[r * 4 + 3];
    double U[9], s[3], V[9];
    svd3_host(A, U, s, V);
    *min_sv = s[2];
    double R[9];
    auto make_R = [&]() {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) R[r * 3 + c] = U[r * 3] * V[c * 3] + U[r * 3 + 1] * V[c * 3 + 1] + U[r * 3 + 2] * V[c * 3 + 2];
    };
    make_R();
    if (det3(R) < 0) {  // mirrored: R stays a proper rotation, the flip goes into S
        for (int r = 0; r < 3; ++r) U[r * 3 + 2] = -U[r * 3 + 2];
        s[2] = -s[2];
        make_R();
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) S[r * 3 + c] = V[r * 3] * s[0] * V[c * 3] + V[r * 3 + 1] * s[1] * V[c * 3 + 1] + V[r * 3 + 2] * s[2] * V[c * 3 + 2];
    // quaternion: magnitudes from the diagonal, signs from the antisymmetric part (mpm_core/geometry.py:42-50)
    double w = std::sqrt(std::max(0.0, 1 + R[0] + R[4] + R[8])) / 2;
    double x = std::copysign(std::sqrt(std::max(0.0, 1 + R[0] - R[4] - R[8])) / 2, R[7] - R[5]);
    double y = std::copysign(std::sqrt(std::max(0.0, 1 - R[0] + R[4] - R[8])) / 2, R[2] - R[6]);
    double z = std::copysign(std::sqrt(std::max(0.0, 1 - R[0] - R[4] + R[8])) / 2, R[3] - R[1]);
    double nq = std::sqrt(x * x + y * y + z * z + w * w);
    q[0] = x / nq; q[1] = y / nq; q[2] = z / nq; q[3] = w / nq;
}


// Static collider fields (warp/solver.py:142-150): flags, local bounding box, offsets of its BVH data.
inline void collider_static(ColliderDev& col, const MpmColliderDesc& d, int node_offset, int tri_offset) {
    col = ColliderDev{};
    col.closed = d.closed ? 1 : 0;
    col.friction = (float)d.friction;
    col.node_offset = node_offset;
    col.tri_offset = tri_offset;
    col.n_tris = d.n_tris;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < d.n_verts; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], d.verts[3 * i + a]);
            hi[a] = std::max(hi[a], d.verts[3 * i + a]);
        }
    col.mesh_scale = 0.0f;
    for (int a = 0; a < 3; ++a) {
        col.aabb_lo[a] = lo[a];
        col.aabb_hi[a] = hi[a];
        if (d.n_verts > 0) col.mesh_scale = std::max({col.mesh_scale, std::fabs(lo[a]), std::fabs(hi[a])});
    }
}

// Pose pair of the next advance (warp/solver.py:154-172): decomposed start and end matrices, the end
// quaternion flipped to the short way round, and the bounding-box margin of three cells in local units
// under the strongest shrink of either pose.
inline void collider_set_pose(ColliderDev& col, const float* start16, const float* end16, double dx) {
    double t0[3], q0[4], S0[9], t1[3], q1[4], S1[9], sv0, sv1;
    decompose(start16, t0, q0, S0, &sv0);
    decompose(end16, t1, q1, S1, &sv1);
    if (q0[0] * q1[0] + q0[1] * q1[1] + q0[2] * q1[2] + q0[3] * q1[3] < 0)
        for (double& v : q1) v = -v;
    for (int k = 0; k < 3; ++k) { col.t0[k] = (float)t0[k]; col.t1[k] = (float)t1[k]; }
    for (int k = 0; k < 4; ++k) { col.q0[k] = (float)q0[k]; col.q1[k] = (float)q1[k]; }
    for (int k = 0; k < 9; ++k) { col.S0[k] = (float)S0[k]; col.S1[k] = (float)S1[k]; }
    double inv_scale = std::max(1.0 / std::max(sv0, 1e-12), 1.0 / std::max(sv1, 1e-12));
    col.margin = (float)(3.0 * dx * inv_scale);
}

// Extent and resolution of a collider's narrow-band voxel grid. It covers the local bounding box grown by
// 1.25 x the margin the current poses need, with a contact cutoff of 1.25 x one grid cell in local units,
// so small changes of scale from frame to frame do not force a rebuild. Voxels are half the cutoff wide,
// at most about 193 per axis: a voxel lists the triangles within its centre's distance plus its diameter,
// so halving the voxel roughly halves the lists near the surface (the 5,120-triangle sphere of the mixed
// workload: 21 instead of 52 candidates within a grid cell of the surface, at most 89 instead of 128 or
// the BVH walk three cells inside), at 8 times the voxels.
inline void sdf_grid_params(ColliderDev& col, int64_t cell_offset) {
    SdfGridDev& g = col.sdf;
    const double margin = 1.25 * col.margin;
    const double cutoff = 1.25 * col.margin / 3.0;  // margin is three grid cells at the strongest shrink
    double extent_max = 0.0, extent[3];
    for (int a = 0; a < 3; ++a) {
        extent[a] = (double)col.aabb_hi[a] - col.aabb_lo[a] + 2.0 * margin;
        extent_max = std::max(extent_max, extent[a]);
    }
    const double hv = std::max(0.5 * cutoff, extent_max / 192.0);
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = (float)(col.aabb_lo[a] - margin);
        g.dims[a] = std::max(1, (int)std::ceil(extent[a] / hv) + 1);
    }
    g.h = (float)hv;
    g.cutoff = (float)cutoff;
    g.thick = (float)(2.0 * cutoff);  // the open-mesh thickness is two grid cells
    g.margin = (float)margin;
    g.built = 0;
    g.cell_offset = cell_offset;
}

}  // namespace mpm

// Host build of the backend's device math (mpm_device.cuh) and BVH builder (mpm_bvh.h), so the CPU test
// suite can check the SVD's accuracy and the BVH closest-point query against the oracle without a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../mpm_plugin_gb300/csrc/mpm_bvh.h"
#include "../../mpm_plugin_gb300/csrc/mpm_device.cuh"

using namespace mpm;

extern "C" {

// The G2P path of the SVD: the FP32 sweeps started from the basis of quaternion Q (4 per matrix, x y z w),
// no FP64 fallback; the new basis back as a quaternion to Qout. Returns how many lanes did not converge.
int svd_warm_batch(int n, const float* A, const float* Q, float* U, float* s, float* d, float* V, float* Qout) {
    unsigned int missed = 0;
    for (int k = 0; k < n; ++k) {
        float a[3][3], u[3][3], v[3][3], v0[3][3];
        for (int i = 0; i < 9; ++i) a[i / 3][i % 3] = A[9 * k + i];
        quat_to_rotation(&Q[4 * k], v0);
        svd3<false>(a, u, &s[3 * k], &d[3 * k], v, &missed, v0);
        rotation_to_quat(v, &Qout[4 * k]);
        for (int i = 0; i < 9; ++i) {
            U[9 * k + i] = u[i / 3][i % 3];
            V[9 * k + i] = v[i / 3][i % 3];
        }
    }
    return (int)missed;
}

// n row-major 3x3 matrices -> U, sigma, d = sigma - 1, V; returns how many lanes took the FP64 path
int svd_batch(int n, const float* A, float* U, float* s, float* d, float* V) {
    unsigned int fp64 = 0;
    for (int k = 0; k < n; ++k) {
        float a[3][3], u[3][3], v[3][3];
        for (int i = 0; i < 9; ++i) a[i / 3][i % 3] = A[9 * k + i];
        svd3(a, u, &s[3 * k], &d[3 * k], v, &fp64);
        for (int i = 0; i < 9; ++i) {
            U[9 * k + i] = u[i / 3][i % 3];
            V[9 * k + i] = v[i / 3][i % 3];
        }
    }
    return (int)fp64;
}

void stress_batch(int n, int model, const float* F, float mu, float lam, float* tau) {
    for (int k = 0; k < n; ++k) {
        float f[3][3], t[3][3];
        for (int i = 0; i < 9; ++i) f[i / 3][i % 3] = F[9 * k + i];
        if (model == 1 || model == 2)
            hencky_tau(f, mu, lam, t, nullptr);
        else
            fixed_corotated_tau(f, mu, lam, t, nullptr);
        for (int i = 0; i < 9; ++i) tau[9 * k + i] = t[i / 3][i % 3];
    }
}

struct HostMesh {
    std::vector<BvhNode> nodes;
    std::vector<MeshTri> tris;
};

void* mesh_build(int nv, const float* verts, int nt, const int32_t* tris) {
    HostMesh* m = new HostMesh();
    build_mesh(MeshInput{nv, nt, verts, tris}, m->nodes, m->tris);
    return m;
}

void mesh_free(void* m) { delete static_cast<HostMesh*>(m); }

// closest point, sign and original face of each query point (local space)
void mesh_query(void* mh, int n, const float* pts, float* cp, float* sign, int32_t* face) {
    HostMesh* m = static_cast<HostMesh*>(mh);
    for (int k = 0; k < n; ++k) {
        ColliderDev c{};
        for (const MeshTri& t : m->tris)
            for (int a = 0; a < 3; ++a)
                c.mesh_scale = std::max({c.mesh_scale, std::fabs(t.a[a]), std::fabs(t.b[a]), std::fabs(t.c[a])});
        MeshHit h = mesh_closest(m->nodes.data(), m->tris.data(), &pts[3 * k], query_tol(c, &pts[3 * k]));
        for (int a = 0; a < 3; ++a) cp[3 * k + a] = h.tri >= 0 ? h.cp[a] : 0.f;
        sign[k] = h.sign;
        face[k] = h.tri >= 0 ? m->tris[h.tri].face : -1;
    }
}

}  // extern "C"

// ---- the whole substep of the CUDA backend, run on the host with the same per-item functions ----------
#include "../../mpm_plugin_gb300/csrc/mpm_host.h"
#include "../../mpm_plugin_gb300/csrc/mpm_substep.cuh"

struct Emu {
    GridDesc g;
    HostDomain hd;
    std::vector<Material> mats;
    std::vector<float4> grid;
    std::vector<ColliderDev> cols;
    std::vector<BvhNode> nodes;
    std::vector<MeshTri> tris;
    std::vector<int2> cells;
    std::vector<int32_t> cand;
    bool use_sdf = true;
    unsigned int fp64 = 0;
};


// Narrow-band voxel grids, built with the same per-voxel functions the GPU build runs.
static void emu_build_sdf(Emu* e) {
    e->cells.clear();
    e->cand.clear();
    int64_t total = 0;
    for (auto& col : e->cols) {
        sdf_grid_params(col, total);
        if (col.n_tris == 0) continue;
        const int64_t nv = (int64_t)col.sdf.dims[0] * col.sdf.dims[1] * col.sdf.dims[2];
        total += nv;
        const BvhNode* nodes = e->nodes.data() + col.node_offset;
        const MeshTri* tris = e->tris.data() + col.tri_offset;
        for (int64_t v = 0; v < nv; ++v) {
            float R2;
            int c = sdf_voxel_classify(col, nodes, tris, v, 128, &R2);
            int start = (int)e->cand.size();
            e->cells.push_back(int2{start, c});
            if (c > 0) {
                float ctr[3], r;
                sdf_voxel_center(col.sdf, v, ctr, &r);
                e->cand.resize(start + c);
                tris_within(nodes, tris, ctr, R2, e->cand.data() + start, c);
            }
        }
        col.sdf.built = 1;
    }
}

extern "C" {

void* emu_create(const MpmDomainDesc* dom, const MpmMaterialDesc* mats, int n_mat, const double* gravity, int ppc) {
    Emu* e = new Emu();
    e->g = make_grid(*dom, gravity, ppc, &e->hd);
    for (int m = 0; m < n_mat; ++m) {
        double wave;
        e->mats.push_back(make_material(mats[m], e->hd.p_vol, &wave));
    }
    e->grid.assign((size_t)e->g.nb[0] * e->g.nb[1] * e->g.nb[2] * 64, float4{0, 0, 0, 0});
    return e;
}

void emu_destroy(void* e) { delete static_cast<Emu*>(e); }

void emu_set_colliders(void* ev, int n, const MpmColliderDesc* cs) {
    Emu* e = static_cast<Emu*>(ev);
    e->cols.assign(n, ColliderDev{});
    e->nodes.clear();
    e->tris.clear();
    for (int c = 0; c < n; ++c) {
        collider_static(e->cols[c], cs[c], (int)e->nodes.size(), (int)e->tris.size());
        std::vector<BvhNode> nd;
        std::vector<MeshTri> tr;
        build_mesh(MeshInput{cs[c].n_verts, cs[c].n_tris, cs[c].verts, cs[c].tris}, nd, tr);
        e->nodes.insert(e->nodes.end(), nd.begin(), nd.end());
        e->tris.insert(e->tris.end(), tr.begin(), tr.end());
    }
}

void emu_set_transforms(void* ev, int n, const float* s16, const float* e16) {
    Emu* e = static_cast<Emu*>(ev);
    for (int c = 0; c < n; ++c) collider_set_pose(e->cols[c], s16 + 16 * c, e16 + 16 * c, e->hd.dx);
    if (e->use_sdf) emu_build_sdf(e);
}

void emu_use_sdf(void* ev, int on) { static_cast<Emu*>(ev)->use_sdf = on != 0; }
void emu_grid_dims(void* ev, int* dims) {
    Emu* e = static_cast<Emu*>(ev);
    for (int a = 0; a < 3; ++a) dims[a] = e->g.dims[a];
}

// Stored-stress form of particles from F (9, n) planar, Jp and mat: tau (6, n) planar.
void emu_particle_stress(void* ev, int64_t n, float* F, float* Jp, int32_t* mat, float* tau) {
    Emu* e = static_cast<Emu*>(ev);
    Particles P{};
    for (int k = 0; k < 9; ++k) P.F[k] = F + k * n;
    for (int k = 0; k < 6; ++k) P.tau[k] = tau + k * n;
    P.Jp = Jp;
    P.mat = mat;
    P.n = P.cap = n;
    for (int64_t p = 0; p < n; ++p) particle_stress(P, p, e->mats.data(), &e->fp64);
}

// x, v: (3, n) planar; C, F: (9, n) planar row-major components; tau: (6, n) stored stress, computed from
// F and Jp first when stress_valid is 0 (particles that just entered); Jp, mat: (n)
unsigned int emu_substep(void* ev, int64_t n, float* x, float* v, float* C, float* F, float* Jp, float* tau,
                         int stress_valid, int32_t* mat, double dt, double s, double frame_dt) {
    Emu* e = static_cast<Emu*>(ev);
    Particles P{};
    for (int a = 0; a < 3; ++a) { P.x[a] = x + a * n; P.v[a] = v + a * n; }
    for (int k = 0; k < 9; ++k) { P.C[k] = C + k * n; P.F[k] = F + k * n; }
    P.Jp = Jp;
    for (int k = 0; k < 6; ++k) P.tau[k] = tau + k * n;
    P.mat = mat;
    // the SVD bases G2P starts from: the identity, or those of the stress computed below
    std::vector<float> vq(4 * (size_t)n, 0.0f);
    for (int64_t p = 0; p < n; ++p) vq[3 * (size_t)n + p] = 1.0f;
    for (int k = 0; k < 4; ++k) P.Vq[k] = vq.data() + k * n;
    P.n = n;
    P.cap = n;
    if (!stress_valid)
        for (int64_t p = 0; p < n; ++p) particle_stress(P, p, e->mats.data(), &e->fp64);
    const float dtf = (float)dt;
    std::vector<ColliderPose> poses(e->cols.size());
    for (size_t c = 0; c < e->cols.size(); ++c) collider_pose_at(e->cols[c], (float)s, (float)(1.0 / frame_dt), poses[c]);
    std::fill(e->grid.begin(), e->grid.end(), float4{0, 0, 0, 0});
    ColliderData cd{};
    cd.cols = e->cols.empty() ? nullptr : e->cols.data();
    cd.poses = poses.empty() ? nullptr : poses.data();
    cd.n_col = (int)e->cols.size();
    cd.nodes = e->nodes.data();
    cd.tris = e->tris.data();
    cd.cells = e->use_sdf && !e->cells.empty() ? e->cells.data() : nullptr;
    cd.cand = e->cand.empty() ? nullptr : e->cand.data();
    const int n_col = cd.n_col;
    for (int64_t p = 0; p < n; ++p) p2g_particle(P, p, e->mats.data(), e->g, dtf, e->grid.data());
    const int64_t nblk = (int64_t)e->g.nb[0] * e->g.nb[1] * e->g.nb[2];
    for (int64_t blk = 0; blk < nblk; ++blk) {
        const int bk = (int)(blk % e->g.nb[2]), bj = (int)((blk / e->g.nb[2]) % e->g.nb[1]);
        const int bi = (int)(blk / ((int64_t)e->g.nb[2] * e->g.nb[1]));
        for (int l = 0; l < 64; ++l) {
            const int idx[3] = {bi * 4 + (l >> 4), bj * 4 + ((l >> 2) & 3), bk * 4 + (l & 3)};
            float4* node = &e->grid[blk * 64 + l];
            if (!grid_node_walls(e->g, node, idx, dtf) || n_col == 0) continue;
            float pos[3];
            node_position(e->g, idx, pos);
            if (near_any_collider(pos, cd)) grid_node_colliders(e->g, node, idx, cd);
        }
    }
    for (int64_t p = 0; p < n; ++p) {
        float nx[3];
        g2p_particle(P, p, e->mats.data(), e->g, dtf, e->grid.data(), &e->fp64, nx);
        if (n_col > 0 && near_any_collider(nx, cd)) project_particle(P, p, e->g, cd);
    }
    return e->fp64;
}

// collider_sdf of collider c at substep fraction s for n world points: out (n, 4) = normal, phi
void emu_collider_sdf(void* ev, int c, float s, int use_sdf, int n, const float* pts, float* out) {
    Emu* e = static_cast<Emu*>(ev);
    ColliderPose pose;
    collider_pose_at(e->cols[c], s, 1.0f, pose);
    const int2* cells = use_sdf && !e->cells.empty() ? e->cells.data() : nullptr;
    const int32_t* cand = e->cand.empty() ? nullptr : e->cand.data();
    for (int k = 0; k < n; ++k) {
        float nn[3], phi = 1.0e30f;
        if (in_margin_box(e->cols[c], pose, &pts[3 * k]))
            collider_sdf(e->cols[c], pose, e->nodes.data(), e->tris.data(), cells, cand, &pts[3 * k], e->g.thickness, nn,
                         &phi);
        else
            nn[0] = nn[1] = 0.f, nn[2] = 1.f;
        out[4 * k] = nn[0]; out[4 * k + 1] = nn[1]; out[4 * k + 2] = nn[2]; out[4 * k + 3] = phi;
    }
}

// Narrow-band voxel grid of collider c as built: desc = lo (3), voxel edge, contact cutoff, dims (3); cells
// (n, 2) = first candidate, count (or kSdfFar / kSdfUseBvh) when cap >= n. Returns the voxel count n.
int64_t emu_sdf_cells(void* ev, int c, float* desc, int32_t* cells, int64_t cap) {
    Emu* e = static_cast<Emu*>(ev);
    const SdfGridDev& g = e->cols[c].sdf;
    for (int a = 0; a < 3; ++a) { desc[a] = g.lo[a]; desc[5 + a] = (float)g.dims[a]; }
    desc[3] = g.h;
    desc[4] = g.cutoff;
    const int64_t n = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
    if (cells && cap >= n && g.built)
        for (int64_t v = 0; v < n; ++v) {
            cells[2 * v] = e->cells[g.cell_offset + v].x;
            cells[2 * v + 1] = e->cells[g.cell_offset + v].y;
        }
    return n;
}

// The C++ host decomposition of a world matrix (mpm_host.h decompose): t (3), q (4, x y z w), S (9)
void host_decompose(const float* m16, double* t, double* q, double* S) {
    double min_sv;
    decompose(m16, t, q, S, &min_sv);
}

// The collider pose the kernels use at substep fraction s for the pose pair (start, end): M (12, 3x4)
void host_collider_matrix(const float* start16, const float* end16, double dx, float s, float* M12) {
    ColliderDev col{};
    collider_set_pose(col, start16, end16, dx);
    ColliderPose pose;
    collider_pose_at(col, s, 1.0f, pose);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) M12[r * 4 + c] = pose.M[r][c];
}

// The FP32 return-mapping projections of n singular-value triples (sig = 1 + d): model 2 Drucker-Prager with
// p = (mu, lam, alpha), model 3 snow with p = (clamp_lo, clamp_hi); out delta (n, 3), whether the projection
// changed the triple and whether the call reported its decision as marginal (n each)
void host_project(int model, int n, const float* sig, const float* d, const float* p, float* delta, int* changed,
                  int* marginal) {
    for (int k = 0; k < n; ++k) {
        bool m = true, c;
        if (model == 2) {
            c = project_drucker_prager(&sig[3 * k], &d[3 * k], p[0], p[1], p[2], &delta[3 * k], &m);
        } else {
            float jp;
            c = project_snow(&sig[3 * k], &d[3 * k], p[0], p[1], &delta[3 * k], &jp, &m);
        }
        changed[k] = c;
        marginal[k] = m;
    }
}

void emu_read_grid(void* ev, float* out) {
    Emu* e = static_cast<Emu*>(ev);
    const GridDesc& g = e->g;
    int64_t q = 0;
    for (int i = 0; i < g.dims[0]; ++i)
        for (int j = 0; j < g.dims[1]; ++j)
            for (int k = 0; k < g.dims[2]; ++k, ++q) {
                float4 v = e->grid[node_index(g, i, j, k)];
                out[4 * q] = v.x; out[4 * q + 1] = v.y; out[4 * q + 2] = v.z; out[4 * q + 3] = v.w;
            }
}

}  // extern "C"

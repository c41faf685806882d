// Host build of the backend's device math (mpm_device.cuh) and BVH builder (mpm_bvh.h), so the CPU test
// suite can check the SVD's accuracy and the BVH closest-point query against the oracle without a GPU.
#include <cuda_runtime.h>

#include <vector>

#include "../../mpm_plugin_gb300/csrc/mpm_bvh.h"
#include "../../mpm_plugin_gb300/csrc/mpm_device.cuh"

using namespace mpm;

extern "C" {

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

// Host-side construction of a collider's BVH and per-triangle query data (local space, built once per
// set_colliders). Header-only and free of CUDA API calls, so tests can build the same structures on the CPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "mpm_types.h"

namespace mpm {

struct MeshInput {
    int n_verts, n_tris;
    const float* verts;   // (n_verts, 3)
    const int32_t* tris;  // (n_tris, 3)
};

inline float round_down(double v) {
    float f = (float)v;
    return (double)f > v ? std::nextafter(f, -INFINITY) : f;
}
inline float round_up(double v) {
    float f = (float)v;
    return (double)f < v ? std::nextafter(f, INFINITY) : f;
}

struct BvhBuilder {
    const float* verts;
    const int32_t* tris;
    std::vector<double> cent;
    std::vector<int> order;
    std::vector<BvhNode> nodes;

    void build(int node, int start, int count) {
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = start; i < start + count; ++i) {
            int t = order[i];
            for (int c = 0; c < 3; ++c)
                for (int a = 0; a < 3; ++a) {
                    double v = verts[3 * tris[3 * t + c] + a];
                    lo[a] = std::min(lo[a], v);
                    hi[a] = std::max(hi[a], v);
                }
            for (int a = 0; a < 3; ++a) {
                clo[a] = std::min(clo[a], cent[3 * t + a]);
                chi[a] = std::max(chi[a], cent[3 * t + a]);
            }
        }
        for (int a = 0; a < 3; ++a) {
            nodes[node].lo[a] = round_down(lo[a]);
            nodes[node].hi[a] = round_up(hi[a]);
        }
        if (count <= 4) {
            nodes[node].start = start;
            nodes[node].count = count;
            return;
        }
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        std::stable_sort(order.begin() + start, order.begin() + start + count,
                         [&](int a, int b) { return cent[3 * a + axis] < cent[3 * b + axis]; });
        int child = (int)nodes.size();
        nodes.push_back(BvhNode{});
        nodes.push_back(BvhNode{});
        nodes[node].start = child;
        nodes[node].count = 0;
        int half = count / 2;
        build(child, start, half);
        build(child + 1, start + half, count - half);
    }
};

inline void mesh_tris(const MeshInput& c, const std::vector<int>& order, std::vector<MeshTri>& out) {
    const int nt = c.n_tris;
    std::vector<double> fn(3 * (size_t)nt), vn(3 * (size_t)c.n_verts, 0.0);
    auto vert = [&](int i, int a) { return (double)c.verts[3 * i + a]; };
    for (int f = 0; f < nt; ++f) {
        int a = c.tris[3 * f], b = c.tris[3 * f + 1], cc = c.tris[3 * f + 2];
        double e1[3], e2[3];
        for (int k = 0; k < 3; ++k) { e1[k] = vert(b, k) - vert(a, k); e2[k] = vert(cc, k) - vert(a, k); }
        double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double l = std::max(std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), 1e-300);
        for (int k = 0; k < 3; ++k) fn[3 * f + k] = n[k] / l;
    }
    // edge pseudonormals: sum of the unit normals of every face on the undirected edge
    struct E { int lo, hi, face, slot; };
    std::vector<E> edges;
    edges.reserve(3 * (size_t)nt);
    for (int f = 0; f < nt; ++f)
        for (int s = 0; s < 3; ++s) {
            int a = c.tris[3 * f + s], b = c.tris[3 * f + (s + 1) % 3];
            edges.push_back({std::min(a, b), std::max(a, b), f, s});
        }
    std::sort(edges.begin(), edges.end(), [](const E& x, const E& y) {
        return x.lo != y.lo ? x.lo < y.lo : (x.hi != y.hi ? x.hi < y.hi : x.face < y.face);
    });
    std::vector<double> en(9 * (size_t)nt, 0.0);
    for (size_t i = 0; i < edges.size();) {
        size_t j = i;
        double sum[3] = {0, 0, 0};
        while (j < edges.size() && edges[j].lo == edges[i].lo && edges[j].hi == edges[i].hi) {
            for (int k = 0; k < 3; ++k) sum[k] += fn[3 * edges[j].face + k];
            ++j;
        }
        for (size_t q = i; q < j; ++q)
            for (int k = 0; k < 3; ++k) en[9 * edges[q].face + 3 * edges[q].slot + k] = sum[k];
        i = j;
    }
    // vertex pseudonormals: face normals weighted by the face's angle at the vertex
    for (int f = 0; f < nt; ++f)
        for (int s = 0; s < 3; ++s) {
            int v0 = c.tris[3 * f + s], v1 = c.tris[3 * f + (s + 1) % 3], v2 = c.tris[3 * f + (s + 2) % 3];
            double e1[3], e2[3];
            for (int k = 0; k < 3; ++k) { e1[k] = vert(v1, k) - vert(v0, k); e2[k] = vert(v2, k) - vert(v0, k); }
            double den = std::max(std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]) *
                                      std::sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]), 1e-300);
            double ca = std::min(1.0, std::max(-1.0, (e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]) / den));
            double ang = std::acos(ca);
            for (int k = 0; k < 3; ++k) vn[3 * v0 + k] += ang * fn[3 * f + k];
        }
    for (int t : order) {
        MeshTri m{};
        const int32_t* tri = &c.tris[3 * t];
        for (int k = 0; k < 3; ++k) {
            m.a[k] = c.verts[3 * tri[0] + k];
            m.b[k] = c.verts[3 * tri[1] + k];
            m.c[k] = c.verts[3 * tri[2] + k];
            m.fn[k] = (float)fn[3 * t + k];
        }
        m.face = t;
        for (int s = 0; s < 3; ++s)
            for (int k = 0; k < 3; ++k) {
                m.en[s][k] = (float)en[9 * t + 3 * s + k];
                m.vn[s][k] = (float)vn[3 * tri[s] + k];
            }
        out.push_back(m);
    }
}


// Builds the BVH (children of an internal node are adjacent; leaves hold up to 4 triangles) and the
// leaf-ordered triangle records of one mesh.
inline void build_mesh(const MeshInput& m, std::vector<BvhNode>& nodes, std::vector<MeshTri>& tris) {
    BvhBuilder b;
    b.verts = m.verts;
    b.tris = m.tris;
    b.cent.resize(3 * (size_t)m.n_tris);
    b.order.resize(m.n_tris);
    for (int t = 0; t < m.n_tris; ++t) {
        b.order[t] = t;
        for (int a = 0; a < 3; ++a)
            b.cent[3 * t + a] = ((double)m.verts[3 * m.tris[3 * t] + a] + m.verts[3 * m.tris[3 * t + 1] + a] +
                                 m.verts[3 * m.tris[3 * t + 2] + a]) / 3.0;
    }
    b.nodes.push_back(BvhNode{});
    if (m.n_tris > 0) {
        b.build(0, 0, m.n_tris);
    } else {  // empty mesh: one empty node that no query can reach
        for (int a = 0; a < 3; ++a) { b.nodes[0].lo[a] = INFINITY; b.nodes[0].hi[a] = -INFINITY; }
    }
    nodes = b.nodes;
    tris.clear();
    mesh_tris(m, b.order, tris);
}

}  // namespace mpm

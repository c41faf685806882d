// Marching-cubes case table, built on the host from the cube's geometry instead of stored as literals.
//
// Corners: c = x + 2 y + 4 z (x, y, z in {0, 1}). Edges: e = 4 a + s runs along axis a from the corner with
// coordinate 0 on a to the one with 1; s = u + 2 w holds the corner's coordinates on the other two axes in
// cyclic order (a + 1) % 3, (a + 2) % 3. A corner is inside when its field value is above the iso level.
//
// Per case (the 8 inside bits), every face contributes directed segments between the edge crossings on its
// border: walking the face's corners counter-clockwise about its outward normal, each run of inside corners
// starts at an entry crossing (outside -> inside) and ends at an exit crossing; the segment goes from entry
// to exit. On a face with two diagonal inside corners each corner is its own run (the inside corners stay
// separate), a choice that depends only on the face's four corners, so the two cells sharing a face draw
// the same segments in opposite directions and the mesh has no cracks. Every crossing edge is the entry of
// one segment and the exit of another, so the segments close into loops; each loop (started at its lowest
// edge) is cut into a fan of triangles whose winding puts the inside (field above iso) behind them: the
// normals point outward. The fan's apex is the first loop vertex from which no triangle has all three
// vertices on one face (such a triangle would be drawn again, reversed, by the neighbouring cell).
#pragma once

#include <cstdint>

namespace mpm {

constexpr int kMcMaxTris = 12;  // at most 12 crossings per cube, so at most 12 - 2 fan triangles

struct McTable {
    int8_t ntri[256];
    int8_t edge[256][kMcMaxTris * 3];  // triangle t of case m: edges edge[m][3 t .. 3 t + 2]
};

// Corner at coordinates (x, y, z).
inline int mc_corner(int x, int y, int z) { return x + 2 * y + 4 * z; }

// The two corners of edge e: along axis a, the other axes' coordinates from s.
inline void mc_edge_corners(int e, int* ca, int* cb) {
    const int a = e >> 2, s = e & 3, u = (a + 1) % 3, w = (a + 2) % 3;
    int lo[3] = {0, 0, 0};
    lo[u] = s & 1;
    lo[w] = s >> 1;
    int hi[3] = {lo[0], lo[1], lo[2]};
    hi[a] = 1;
    *ca = mc_corner(lo[0], lo[1], lo[2]);
    *cb = mc_corner(hi[0], hi[1], hi[2]);
}

// Bit set of the two faces an edge lies on: face 2 a + side.
inline int mc_edge_faces(int e) {
    const int a = e >> 2, s = e & 3, u = (a + 1) % 3, w = (a + 2) % 3;
    return (1 << (2 * u + (s & 1))) | (1 << (2 * w + (s >> 1)));
}

// The edge joining corners p and q (which differ in one coordinate).
inline int mc_edge_of(int p, int q) {
    for (int e = 0; e < 12; ++e) {
        int a, b;
        mc_edge_corners(e, &a, &b);
        if ((a == p && b == q) || (a == q && b == p)) return e;
    }
    return -1;
}

inline McTable build_mc_table() {
    McTable t{};
    for (int m = 0; m < 256; ++m) {
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int a = 0; a < 3; ++a) {
            const int u = (a + 1) % 3, w = (a + 2) % 3;
            for (int side = 0; side < 2; ++side) {
                // counter-clockwise about the outward normal: (0,0),(1,0),(1,1),(0,1) in (u, w) for +a,
                // the reverse for -a
                const int uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
                int q[4];
                for (int i = 0; i < 4; ++i) {
                    const int k = side ? i : (4 - i) % 4;
                    int c[3];
                    c[a] = side;
                    c[u] = uv[k][0];
                    c[w] = uv[k][1];
                    q[i] = mc_corner(c[0], c[1], c[2]);
                }
                int entry = -1, first_exit = -1;
                for (int i = 0; i < 4; ++i) {
                    const int p = q[i], r = q[(i + 1) & 3];
                    const bool pin = (m >> p) & 1, rin = (m >> r) & 1;
                    if (!pin && rin) entry = mc_edge_of(p, r);
                    if (pin && !rin) {
                        const int ex = mc_edge_of(p, r);
                        if (entry >= 0) {
                            next[entry] = ex;
                            entry = -1;
                        } else {
                            first_exit = ex;  // its run began before q[0]: closed by the last entry
                        }
                    }
                }
                if (entry >= 0 && first_exit >= 0) next[entry] = first_exit;
            }
        }
        bool seen[12] = {};
        int nt = 0;
        for (int e0 = 0; e0 < 12; ++e0) {
            if (next[e0] < 0 || seen[e0]) continue;
            int loop[12], len = 0;
            for (int e = e0; !seen[e]; e = next[e]) {
                seen[e] = true;
                loop[len++] = e;
            }
            int r = 0;  // apex: first rotation without a triangle inside one face
            for (; r < len; ++r) {
                bool ok = true;
                for (int i = 1; i + 1 < len && ok; ++i)
                    ok = !(mc_edge_faces(loop[r]) & mc_edge_faces(loop[(r + i) % len]) &
                           mc_edge_faces(loop[(r + i + 1) % len]));
                if (ok) break;
            }
            if (r == len) r = 0;  // not reached for any of the 256 cases
            for (int i = 1; i + 1 < len; ++i) {
                t.edge[m][3 * nt] = (int8_t)loop[r];
                t.edge[m][3 * nt + 1] = (int8_t)loop[(r + i) % len];
                t.edge[m][3 * nt + 2] = (int8_t)loop[(r + i + 1) % len];
                ++nt;
            }
        }
        t.ntri[m] = (int8_t)nt;
    }
    return t;
}

}  // namespace mpm

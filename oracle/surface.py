"""CPU restatement of the reference's surfacer (mpm_surface/field.py). TEST INFRASTRUCTURE ONLY.

Only tests/ and the CPU-baseline leg of bench.py import this module, as the checker; the product never does.

* ``rest_density``: field.py:92-101 (the mean kernel sum of a particle lattice over eight offsets);
* ``splat`` / ``normalize`` / ``sample_velocity``: field.py:35-89, in float64 (the device sums in float32);
* ``grid_params``: the host set-up of surface_particles (field.py:104-125): cell, kernel radius, padding,
  origin and node counts;
* ``mc_table`` / ``marching_cubes``: a marching-cubes restatement with the device's conventions (a node is
  inside above iso; one vertex per crossing grid edge, node order then axis order; triangles in cell order,
  wound outward). The reference calls warp's MarchingCubes, a dependency (warp-lang 1.18) that is not
  installed here and whose case table and output order are not in the reference's sources, so the mesh
  itself is not pinned to the reference; the table is built here by an independent construction (corner
  coordinates and face normals, not the device's index arithmetic) and checked against the device's.
"""

from __future__ import annotations

import math
from itertools import product

import numpy as np

BYTES_PER_CELL = 56  # field.py:20


def cubic_kernel(q):
    q = np.asarray(q, np.float64)
    t = 1.0 - q
    return np.where(q < 0.5, 1.0 - 6.0 * q * q + 6.0 * q ** 3, np.where(q < 1.0, 2.0 * t ** 3, 0.0))


def rest_density(spacing: float, h: float) -> float:
    n = math.ceil(h / spacing) + 1
    lattice = np.stack(np.meshgrid(*[np.arange(-n, n + 1)] * 3, indexing="ij"), -1).reshape(-1, 3) * spacing
    sums = []
    for offset in np.array(list(product((0, 0.5), repeat=3))) * spacing:
        q = np.linalg.norm(lattice - offset, axis=1) / h
        sums.append(cubic_kernel(q).sum())
    return float(np.mean(sums))


def grid_params(positions, spacing: float, detail: float, smoothing: float):
    """(origin float64, dims, cell, h) as surface_particles sets them up (field.py:112-117)."""
    positions = np.asarray(positions, np.float32).reshape(-1, 3)
    cell = spacing / detail
    h = 2.0 * spacing * smoothing
    pad = h + 2.0 * cell
    origin = positions.min(0).astype(np.float64) - pad
    dims = tuple(int(math.ceil(e / cell)) + 1 for e in positions.max(0) + pad - origin)
    return origin, dims, cell, h


def splat(x, v, origin32, inv_cell32, cell32, h32, dims):
    """Density (dims) and momentum (dims + (3,)) sums, float64."""
    dens = np.zeros(dims, np.float64)
    mom = np.zeros(dims + (3,), np.float64)
    x = np.asarray(x, np.float32)
    v = np.asarray(v, np.float32).astype(np.float64)
    g_all = (x - np.float32(origin32)).astype(np.float32) * np.float32(inv_cell32)
    r = float(np.float32(h32) * np.float32(inv_cell32))
    for g, vel in zip(g_all.astype(np.float64), v):
        lo = np.maximum(np.floor(g - r).astype(int), 0)
        hi = np.minimum(np.ceil(g + r).astype(int), np.array(dims) - 1)
        if np.any(hi < lo):
            continue
        ii, jj, kk = np.meshgrid(*[np.arange(lo[a], hi[a] + 1) for a in range(3)], indexing="ij")
        d = np.sqrt((ii - g[0]) ** 2 + (jj - g[1]) ** 2 + (kk - g[2]) ** 2) * float(cell32)
        w = cubic_kernel(d / float(h32))
        sel = w > 0
        np.add.at(dens, (ii[sel], jj[sel], kk[sel]), w[sel])
        np.add.at(mom, (ii[sel], jj[sel], kk[sel]), w[sel][:, None] * vel)
    return dens, mom


def normalize(dens, mom, inv_rest):
    vel = np.where(dens[..., None] > 0, mom / np.where(dens > 0, dens, 1.0)[..., None], mom)
    return dens * inv_rest, vel


def sample_velocity(verts, vel):
    dims = np.array(vel.shape[:3])
    base = np.clip(np.floor(verts).astype(int), 0, dims - 2)
    f = verts - base
    out = np.zeros_like(verts, dtype=np.float64)
    for a, b, c in product((0, 1), repeat=3):
        w = (f[:, 0] if a else 1 - f[:, 0]) * (f[:, 1] if b else 1 - f[:, 1]) * (f[:, 2] if c else 1 - f[:, 2])
        out += w[:, None] * vel[base[:, 0] + a, base[:, 1] + b, base[:, 2] + c]
    return out


# ---- marching cubes -----------------------------------------------------------------------------------
CORNERS = np.array([(c & 1, (c >> 1) & 1, c >> 2) for c in range(8)])  # corner c = x + 2 y + 4 z


def _edge_id(p: int, q: int) -> int:
    """Edge 4 a + s between corners p and q: a the axis they differ on, s the lower corner's coordinates on
    the axes (a + 1) % 3 and (a + 2) % 3 as s = u + 2 w."""
    lo = np.minimum(CORNERS[p], CORNERS[q])
    a = int(np.flatnonzero(CORNERS[p] != CORNERS[q])[0])
    return 4 * a + int(lo[(a + 1) % 3]) + 2 * int(lo[(a + 2) % 3])


def _faces(e: int) -> set:
    """The two faces (axis, side) that edge e lies on, from its corners' coordinates."""
    a, s = e >> 2, e & 3
    lo = np.zeros(3, int)
    lo[(a + 1) % 3], lo[(a + 2) % 3] = s & 1, s >> 1
    return {(ax, int(lo[ax])) for ax in range(3) if ax != a}


def mc_table():
    """Case -> list of triangles (edge ids), built from corner coordinates: on every cube face, corners are
    ordered counter-clockwise about the outward normal by angle; each run of inside corners gives a segment
    from its entry crossing to its exit crossing; segments chain into loops, loops into triangle fans whose
    apex is the first loop vertex with no triangle lying in one face."""
    faces = []
    for axis, side in product(range(3), (0, 1)):
        normal = np.zeros(3)
        normal[axis] = 1.0 if side else -1.0
        cs = [c for c in range(8) if CORNERS[c][axis] == side]
        centre = CORNERS[cs].mean(0)
        ref = CORNERS[cs[0]] - centre
        def angle(c):
            d = CORNERS[c] - centre
            return math.atan2(float(np.dot(np.cross(ref, d), normal)), float(np.dot(ref, d)))
        faces.append(sorted(cs, key=angle))
    table = []
    for m in range(256):
        inside = [(m >> c) & 1 for c in range(8)]
        succ = {}
        for ring in faces:
            crossings = []  # (kind, edge) in counter-clockwise order
            for i in range(4):
                p, q = ring[i], ring[(i + 1) % 4]
                if inside[p] != inside[q]:
                    crossings.append(("entry" if inside[q] else "exit", _edge_id(p, q)))
            # rotate so the list starts with an entry; then entries and exits alternate
            while crossings and crossings[0][0] != "entry":
                crossings = crossings[1:] + crossings[:1]
            for k in range(0, len(crossings), 2):
                succ[crossings[k][1]] = crossings[k + 1][1]
        tris, seen = [], set()
        for e0 in sorted(succ):
            if e0 in seen:
                continue
            loop, e = [], e0
            while e not in seen:
                seen.add(e)
                loop.append(e)
                e = succ[e]
            for r in range(len(loop)):
                ring = loop[r:] + loop[:r]
                fan = [(ring[0], ring[i], ring[i + 1]) for i in range(1, len(ring) - 1)]
                if all(not (_faces(a) & _faces(b) & _faces(c)) for a, b, c in fan):
                    break
            tris += fan
        table.append(tris)
    return table


def marching_cubes(dens, iso, table=None):
    """(verts (V, 3) float64 in grid index units, tris (T, 3) int32), the device's conventions."""
    table = table or mc_table()
    dims = dens.shape
    inside = dens > iso
    vid = -np.ones(dims + (3,), np.int64)
    verts = []
    nodes = np.argwhere(np.ones(dims, bool))  # C order
    for (i, j, k) in nodes:
        for a in range(3):
            nb = [i, j, k]
            nb[a] += 1
            if nb[a] >= dims[a] or inside[i, j, k] == inside[tuple(nb)]:
                continue
            d0, d1 = np.float32(dens[i, j, k]), np.float32(dens[tuple(nb)])
            t = (np.float32(iso) - d0) / (d1 - d0)
            p = np.array([i, j, k], np.float64)
            p[a] += float(t)
            vid[i, j, k, a] = len(verts)
            verts.append(p)
    tris = []
    for (i, j, k) in nodes:
        if i + 1 >= dims[0] or j + 1 >= dims[1] or k + 1 >= dims[2]:
            continue
        m = sum(1 << c for c in range(8) if inside[i + CORNERS[c][0], j + CORNERS[c][1], k + CORNERS[c][2]])
        for tri in table[m]:
            ids = []
            for e in tri:
                a, s = e >> 2, e & 3
                o = [0, 0, 0]
                o[(a + 1) % 3] = s & 1
                o[(a + 2) % 3] = s >> 1
                ids.append(vid[i + o[0], j + o[1], k + o[2], a])
            tris.append(ids)
    return np.array(verts, np.float64).reshape(-1, 3), np.array(tris, np.int32).reshape(-1, 3)


def surface_particles(positions, velocities, spacing, detail=1.0, smoothing=2.0, iso=0.35):
    """The whole surfacing of one particle set on the CPU: (verts world float32, tris, vel float32) and the
    intermediate fields (density, velocity) for comparisons."""
    positions = np.asarray(positions, np.float32).reshape(-1, 3)
    origin, dims, cell, h = grid_params(positions, spacing, detail, smoothing)
    dens, mom = splat(positions, velocities, np.float32(origin), np.float32(1.0 / cell), np.float32(cell),
                      np.float32(h), dims)
    dens_n, vel = normalize(dens, mom, float(np.float32(1.0 / rest_density(spacing, h))))
    verts, tris = marching_cubes(dens_n.astype(np.float32), np.float32(iso))
    vv = sample_velocity(verts, vel)
    world = (origin + verts * cell).astype(np.float32)
    return {"verts": world, "tris": tris, "vel": vv.astype(np.float32), "verts_index": verts,
            "density": dens_n, "velocity": vel, "origin": origin, "dims": dims, "cell": cell, "h": h}

"""Seeded synthetic workloads of the measured configurations, built with this package alone.

The benchmark (bench.py) and users who want the same scenes build them here: meshes (box, plane, geodesic
sphere, torus, cylinder), transforms, jittered particle lattices, and mesh volumes sampled on the GPU with
the reference's lattice and jitter (mpm_plugin_gb300.emit.sample_mesh_volume). Scenes:

  mixed_scene     128^3 mixed materials: von Mises sphere, Drucker-Prager column, thrown snowball and a static
                  seeded perturbed geodesic sphere collider of 5,120 triangles;
  jelly_cube      the 64^3 fixed-corotated cube (about 32k particles);
  large_scene     the 256^3 granular pour: pile, turning 20,480-triangle torus, disc inflow;
  batched_scenes  64 independent scenes of log-uniform size, four material models, 0-2 colliders;
  pour_job        one serving request: a pour at a serving size with inflow and a turning torus.
"""

from __future__ import annotations

import numpy as np

from mpm_plugin_gb300.interface import Domain, MaterialParams

WALL_SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")


# -- transforms (4 x 4, float32) -------------------------------------------------------------------------------
def translate(x, y, z) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (x, y, z)
    return m


def scale(x, y=None, z=None) -> np.ndarray:
    return np.diag([x, x if y is None else y, x if z is None else z, 1.0]).astype(np.float32)


def _rot(axis: int, deg: float) -> np.ndarray:
    a, b = [(1, 2), (2, 0), (0, 1)][axis]
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    m = np.eye(4, dtype=np.float32)
    m[a, a], m[a, b], m[b, a], m[b, b] = c, -s, s, c
    return m


def rot_x(deg: float) -> np.ndarray:
    return _rot(0, deg)


def rot_y(deg: float) -> np.ndarray:
    return _rot(1, deg)


def rot_z(deg: float) -> np.ndarray:
    return _rot(2, deg)


def transform_points(m: np.ndarray, pts: np.ndarray) -> np.ndarray:
    m = np.asarray(m, np.float64)
    return (np.asarray(pts, np.float64) @ m[:3, :3].T + m[:3, 3]).astype(np.float32)


# -- meshes (float32 vertices, int32 triangles, outward winding) -------------------------------------------------
def _outward(verts: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """Triangles of a mesh that is star-shaped about the origin, each wound so its normal points away from it."""
    a, b, c = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    flip = (np.cross(b - a, c - a) * (a + b + c)).sum(1) < 0
    tris = tris.copy()
    tris[flip, 1], tris[flip, 2] = tris[flip, 2], tris[flip, 1].copy()
    return tris


def box_mesh(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Closed axis-aligned box (12 triangles)."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    corners = np.array([[(hi if (i >> a) & 1 else lo)[a] for a in range(3)] for i in range(8)])
    quads = [(0, 2, 6, 4), (1, 5, 7, 3), (0, 4, 5, 1), (2, 3, 7, 6), (0, 1, 3, 2), (4, 6, 7, 5)]
    tris = np.array([t for q in quads for t in ((q[0], q[1], q[2]), (q[0], q[2], q[3]))], np.int32)
    centre = (lo + hi) / 2
    return corners.astype(np.float32), _outward(corners - centre, tris)


def plane_mesh(size: float):
    """Open square of side `size` in the xy plane centred at the origin, normal +z."""
    h = size / 2
    return (np.array([[-h, -h, 0], [h, -h, 0], [h, h, 0], [-h, h, 0]], np.float32),
            np.array([[0, 1, 2], [0, 2, 3]], np.int32))


def geodesic_sphere(radius: float, subdivisions: int, seed: int | None = None, jitter: float = 0.0):
    """Sphere of 20 * 4**subdivisions triangles: the 12 vertices (0, +-1, +-phi) and their cyclic permutations,
    the 20 faces found as the vertex triples at the edge length from each other, each face split into four
    per subdivision with its edge midpoints pushed out to the sphere. With a seed every vertex radius is
    scaled by 1 + U(-jitter, jitter)."""
    phi = (1 + 5 ** 0.5) / 2
    base = []
    for s1 in (-1, 1):
        for s2 in (-1, 1):
            base += [(0, s1, s2 * phi), (s1, s2 * phi, 0), (s2 * phi, 0, s1)]
    v = np.array(base, np.float64)
    d2 = ((v[:, None] - v[None]) ** 2).sum(-1)
    edge = np.isclose(d2, 4.0)
    faces = [(i, j, k) for i in range(12) for j in range(i + 1, 12) for k in range(j + 1, 12)
             if edge[i, j] and edge[j, k] and edge[i, k]]
    verts = list(v / np.linalg.norm(v, axis=1, keepdims=True))
    tris = faces
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                cache[key] = len(verts)
                verts.append(m / np.linalg.norm(m))
            return cache[key]

        nxt = []
        for a, b, c in tris:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nxt += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        tris = nxt
    verts = np.array(verts) * radius
    tris = _outward(verts, np.array(tris, np.int32))
    if seed is not None:
        verts = verts * (1 + np.random.default_rng(seed).uniform(-jitter, jitter, (len(verts), 1)))
    return verts.astype(np.float32), tris


def torus(major: float, minor: float, n_major: int, n_minor: int, seed: int | None = None, jitter: float = 0.0):
    """Closed torus around the z axis (2 * n_major * n_minor triangles); with a seed every vertex's tube radius
    is scaled by 1 + U(-jitter, jitter)."""
    u = 2 * np.pi * np.arange(n_major) / n_major
    w = 2 * np.pi * np.arange(n_minor) / n_minor
    r = np.full((n_major, n_minor), minor)
    if seed is not None:
        r = r * (1 + np.random.default_rng(seed).uniform(-jitter, jitter, r.shape))
    cu, su, cw, sw = np.cos(u)[:, None], np.sin(u)[:, None], np.cos(w)[None, :], np.sin(w)[None, :]
    verts = np.stack([(major + r * cw) * cu, (major + r * cw) * su, r * sw], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    a = i * n_minor + j
    b = ((i + 1) % n_major) * n_minor + j
    c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
    d = i * n_minor + (j + 1) % n_minor
    tris = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return verts.astype(np.float32), tris.astype(np.int32)


def cylinder(radius: float, height: float, segments: int = 32):
    """Closed cylinder around the z axis from z = 0 to height (4 * segments triangles, outward winding)."""
    a = 2 * np.pi * np.arange(segments) / segments
    ring = np.stack([radius * np.cos(a), radius * np.sin(a)], -1)
    verts = np.concatenate([np.c_[ring, np.zeros(segments)], np.c_[ring, np.full(segments, height)],
                            [[0.0, 0.0, 0.0], [0.0, 0.0, height]]])
    bc, tc = 2 * segments, 2 * segments + 1
    tris = []
    for k in range(segments):
        k1 = (k + 1) % segments
        tris += [[k, k1, segments + k1], [k, segments + k1, segments + k], [bc, k1, k], [tc, segments + k, segments + k1]]
    return verts.astype(np.float32), np.array(tris, np.int32)


# -- particles and domains ------------------------------------------------------------------------------------
def lattice_box(lo, hi, spacing: float, rng) -> np.ndarray:
    """Particles on a lattice of the given spacing filling [lo, hi], each jittered by U(+-spacing / 4)."""
    axes = [np.arange(lo[a] + spacing / 2, hi[a], spacing, dtype=np.float64) for a in range(3)]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    g += rng.uniform(-0.25 * spacing, 0.25 * spacing, g.shape)
    return g.astype(np.float32)


def sample_volume(verts, tris, spacing: float, seed, device: int = 0) -> np.ndarray:
    """Points inside a closed mesh: the reference's stratified lattice and seeded jitter, sampled on the GPU."""
    from mpm_plugin_gb300.emit import sample_mesh_volume

    return sample_mesh_volume(verts, tris, spacing, seed, device)


def make_domain(res: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), walls=None, wall_friction: float = 0.5) -> Domain:
    return Domain(tuple(lo), tuple(hi), res, {**{s: True for s in WALL_SIDES}, **(walls or {})}, wall_friction)


def cell_size(domain) -> float:
    """Grid spacing of a domain: the longest side over the resolution (mpm_core/scene.py:60-62)."""
    return max(b - a for a, b in zip(domain.min, domain.max)) / domain.resolution


def add_group(solver, positions, material_id: int = 0, emitter_id: int = 0, velocity=(0.0, 0.0, 0.0)) -> None:
    n = len(positions)
    solver.add_particles(positions, np.tile(np.asarray(velocity, np.float32), (n, 1)),
                         np.full(n, material_id, np.int32), np.full(n, emitter_id, np.int32))


# -- scenes ------------------------------------------------------------------------------------------------------
def mixed_scene(res: int = 128, seed: int = 0, device: int = 0, sample=None):
    """Mixed materials in a 1 m box at 8 particles per cell: von Mises sphere r = 0.12 (E 2e4, nu 0.45, yield
    300 Pa, rho 600), Drucker-Prager column 0.15 x 0.4 x 0.15 (E 3.5e5, nu 0.3, 35 deg, rho 1600), snowball
    r = 0.08 thrown at (3, 1, 0) m/s from the -x side (E 1.4e5, nu 0.2, hardening 10, theta_c 2.5e-2,
    theta_s 7.5e-3, max hardening 20, rho 400), and one static seeded perturbed geodesic sphere collider of
    5,120 triangles (radius 0.12 at (0.75, 0.7, 0.1)).
    `sample(verts, tris, spacing, seed)` samples a mesh volume (default: sample_volume on `device`; any sampler
    of the reference's lattice and jitter gives the same points).
    Returns (domain, materials, [(positions, material, velocity)], (collider verts, tris, world matrix))."""
    if sample is None:
        def sample(v, t, spacing, sd):
            return sample_volume(v, t, spacing, sd, device)
    d = make_domain(res)
    dx = cell_size(d)
    mats = [MaterialParams("vm_sphere", "von_mises", 2e4, 0.45, 600.0, yield_stress=300.0),
            MaterialParams("dp_column", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=35.0),
            MaterialParams("snowball", "snow", 1.4e5, 0.2, 400.0, hardening=10.0, critical_compression=2.5e-2,
                           critical_stretch=7.5e-3, max_hardening=20.0)]
    sv, st = geodesic_sphere(1.0, 4)
    sphere = sample(transform_points(translate(0.25, 0.5, 0.3) @ scale(0.12), sv), st, dx / 2, seed)
    bv, bt = box_mesh((0.5, 0.425, 0.0), (0.65, 0.575, 0.4))
    column = sample(bv, bt, dx / 2, seed + 1)
    snow = sample(transform_points(translate(0.2, 0.3, 0.5) @ scale(0.08), sv), st, dx / 2, seed + 2)
    groups = [(sphere, 0, (0.0, 0.0, 0.0)), (column, 1, (0.0, 0.0, 0.0)), (snow, 2, (3.0, 1.0, 0.0))]
    cv, ct = geodesic_sphere(1.0, 4, seed=seed + 3, jitter=0.03)
    return d, mats, groups, (cv, ct, translate(0.75, 0.7, 0.1) @ scale(0.12))


def jelly_cube(res: int = 64, seed: int = 0):
    """The fixed-corotated jelly cube of side 0.25 centred at (0.5, 0.6, 0.5) at 8 per cell (E 1e5, nu 0.3,
    rho 1000, at rest). Returns (domain, materials, positions)."""
    d = make_domain(res)
    mats = [MaterialParams("jelly_cube", "elastic", 1e5, 0.3, 1000.0)]
    pos = lattice_box((0.375, 0.475, 0.375), (0.625, 0.725, 0.625), cell_size(d) / 2, np.random.default_rng(seed))
    return d, mats, pos


def large_scene(res: int, pile_top: float, seed: int = 3):
    """The large inflow workload at resolution `res`: a Drucker-Prager pile (E 3.5e5, nu 0.3, 30 deg,
    rho 1600) filling (0.2-0.8)^2 x (0-pile_top) at 8 per cell, a seeded perturbed torus of 20,480 triangles
    (R 0.2, r 0.05, friction 0.4) turning at 1 rev/s about z, and a disc inflow r = 0.05 m at 2 m/s downward
    (a closed 48-sided cylinder emitter, one emission substep's slab high).
    Returns (domain, materials, pile, torus mesh, pose(t), emit(solver, piece))."""
    d = make_domain(res)
    dx = cell_size(d)
    mats = [MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)]
    pile = lattice_box((0.2, 0.2, 0.0), (0.8, 0.8, pile_top), dx / 2, np.random.default_rng(seed))
    tv, tt = torus(0.2, 0.05, 256, 40, seed=seed, jitter=0.05)

    def pose(t):
        return translate(0.5, 0.5, pile_top + 0.12) @ rot_z(360.0 * t) @ rot_x(90.0)

    ev, et = cylinder(0.05, 2.0 / 96, 48)  # one emission substep's slab of the disc inflow
    ev = ev + np.float32([0.5, 0.5, 0.9])

    def emit(s, piece, device: int = 0):
        """One emission substep as the bake runner's _emit does it for an inflow (bake.py:56-86): the
        emitter volume sampled at spacing dx / 2 with the runner's seed list (seed, frame, emitter 0, the
        substep fraction), points outside the domain dropped, points on occupied nodes dropped, the rest
        added at 2 m/s downward."""
        frame, quarter = divmod(piece, 4)
        pts = sample_volume(ev, et, dx / 2, [seed, frame + 1, 0, quarter + 1, 4], device)
        pts = pts[((pts >= np.asarray(d.min)) & (pts <= np.asarray(d.max))).all(1)]
        if len(pts) and s.particle_count:
            pts = pts[~s.is_occupied(pts)]
        if len(pts):
            add_group(s, pts, velocity=(0.0, 0.0, -2.0))
        return len(pts)

    return d, mats, pile, (tv, tt), pose, emit


BATCH_MODELS = ("elastic", "von_mises", "drucker_prager", "snow")


def batched_scenes(seed: int = 0, count: int = 64, n_lo: float = 1e4, n_hi: float = 2e6):
    """Independent scenes of the batched workload: particle counts log-uniform in [n_lo, n_hi], grids from 32^3
    to 192^3 matched to the count (a cube of material filling the same fraction of every grid, 8 per cell),
    one material per scene with the model uniform over the four and parameters uniform within the ranges of the
    jelly and mixed-materials workloads, a random initial velocity, and 0-2 static seeded perturbed geodesic
    sphere colliders of 1,280, 5,120 or 20,480 triangles below the material.

    Returns [(domain, [material], positions, velocity, [(verts, tris, world matrix, friction)])]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n_target = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        res = int(np.clip(round(32 * (n_target / 1e4) ** (1 / 3)), 32, 192))
        d = make_domain(res)
        side = min((n_target / 8) ** (1 / 3) / res, 0.6)
        lo = (0.5 - side / 2, 0.5 - side / 2, 0.25)
        hi = (0.5 + side / 2, 0.5 + side / 2, 0.25 + side)
        pos = lattice_box(lo, hi, cell_size(d) / 2, rng)
        model = BATCH_MODELS[int(rng.integers(4))]
        mat = MaterialParams(f"batch{i}", model, float(rng.uniform(2e4, 3.5e5)), float(rng.uniform(0.2, 0.45)),
                             float(rng.uniform(400.0, 1600.0)), yield_stress=float(rng.uniform(300.0, 3000.0)),
                             friction_angle_deg=float(rng.uniform(30.0, 35.0)), hardening=10.0,
                             critical_compression=2.5e-2, critical_stretch=7.5e-3,
                             max_hardening=float(rng.uniform(5.0, 20.0)))
        vel = tuple(float(c) for c in rng.uniform(-1.0, 1.0, 3))
        cols = []
        for c in range(int(rng.integers(0, 3))):
            cv, ct = geodesic_sphere(1.0, int(rng.choice([3, 4, 5])), seed=seed * 1000 + i * 10 + c, jitter=0.03)
            r = float(rng.uniform(0.06, 0.12))
            xf = translate(float(rng.uniform(0.25, 0.75)), float(rng.uniform(0.25, 0.75)), r) @ scale(r)
            cols.append((cv, ct, xf, float(rng.uniform(0.0, 0.5))))
        out.append((d, [mat], pos, vel, cols))
    return out


def pour_job(seed: int, res: int = 96, frames: int = 12, fps: float = 24.0, side_range=(0.2, 0.4)):
    """A granular pour (the large inflow workload's distribution at a serving size): a Drucker-Prager pile
    (E 3.5e5, nu 0.3, 30 deg, rho 1600) of seeded size, a disc inflow r = 0.05 m at 2 m/s downward whose slab
    of one frame is added where no material is, and a seeded torus collider (2,048 triangles, friction 0.4)
    turning at 1 rev/s. Returns (domain, materials, setup(solver), before_frame(solver, k), frames, fps,
    max_particles, collider_triangles)."""
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    rng = np.random.default_rng(seed)
    d = make_domain(res)
    dx = cell_size(d)
    mat = MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)
    side = float(rng.uniform(*side_range))
    pile = lattice_box((0.5 - side / 2, 0.5 - side / 2, 0.0), (0.5 + side / 2, 0.5 + side / 2, side / 2), dx / 2,
                       rng)
    tv, tt = torus(0.18, 0.04, 64, 16, seed=seed, jitter=0.05)

    def pose(t):
        return translate(0.5, 0.5, 0.35) @ rot_z(360.0 * t) @ rot_x(90.0)

    def setup(s):
        add_group(s, pile)
        s.set_colliders([ColliderGeometry(MeshData(tv, tt), closed=True, friction=0.4)])

    def before_frame(s, k):
        s.set_collider_transforms(pose((k - 1) / fps)[None], pose(k / fps)[None])
        r = np.random.default_rng(seed * 1000 + k)
        slab = lattice_box((0.45, 0.45, 0.85), (0.55, 0.55, 0.85 + 2.0 / fps), dx / 2, r)
        slab = slab[np.hypot(slab[:, 0] - 0.5, slab[:, 1] - 0.5) <= 0.05]
        free = ~s.is_occupied(slab)
        if free.any():
            add_group(s, slab[free], velocity=(0.0, 0.0, -2.0))

    slab_n = int(np.pi * 0.05 ** 2 * 2.0 / fps * 8 * res ** 3) + 1
    return d, [mat], setup, before_frame, frames, fps, len(pile) + frames * slab_n, len(tt)

"""Seeded test scenes: meshes, particle boxes/spheres, matrices and the reference's material presets.

Particles are sampled with the oracle's restatement of the reference's volume sampler (pinned by the golden
fixtures), so the same seeds give the same particles as the reference's own test helpers.
"""

from __future__ import annotations

import json

import numpy as np
from _golden import GOLDEN, Domain, material_from_dict

from mpm_plugin_gb300.interface import MaterialParams
from oracle import geometry

WALL_SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")
ALL_WALLS = {side: True for side in WALL_SIDES}

_PRESETS = json.loads(str(np.load(GOLDEN / "geometry.npz")["meta"]))["presets"]


def preset(name: str) -> MaterialParams:
    """Material parameters of the reference's built-in preset ``name`` (mpm_core/presets/*.toml)."""
    return material_from_dict(_PRESETS[name]["material"])


def preset_names() -> list[str]:
    return sorted(_PRESETS)


def translate(x, y, z) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (x, y, z)
    return m


def scale(x, y=None, z=None) -> np.ndarray:
    return np.diag([x, x if y is None else y, x if z is None else z, 1.0]).astype(np.float32)


def rot_x(deg: float) -> np.ndarray:
    a = np.radians(deg)
    m = np.eye(4, dtype=np.float32)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = np.cos(a), -np.sin(a), np.sin(a), np.cos(a)
    return m


def rot_y(deg: float) -> np.ndarray:
    a = np.radians(deg)
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = np.cos(a), np.sin(a), -np.sin(a), np.cos(a)
    return m


def unit_cube_mesh(centered: bool = False):
    """Closed cube with outward winding: [0,1]^3, or [-0.5,0.5]^3 when centered."""
    v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32)
    if centered:
        v -= 0.5
    t = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                  [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]], np.int32)
    return v, t


def plane_mesh(size: float):
    """Open square in the xy plane centred at the origin, normal +z."""
    h = size / 2
    return (np.array([[-h, -h, 0], [h, -h, 0], [h, h, 0], [-h, h, 0]], np.float32),
            np.array([[0, 1, 2], [0, 2, 3]], np.int32))


def icosphere(radius: float, subdivisions: int, seed: int | None = None, jitter: float = 0.0):
    """Geodesic sphere by midpoint subdivision of an icosahedron (20 * 4**s triangles, outward winding).

    With a seed, every vertex radius is scaled by 1 + U(-jitter, jitter) (a seeded perturbed sphere).
    """
    p = (1 + 5 ** 0.5) / 2
    verts = [np.array(v, float) for v in ([-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p],
                                          [0, -1, -p], [0, 1, -p], [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1])]
    verts = [v / np.linalg.norm(v) for v in verts]
    faces = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
             [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
             [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    for _ in range(subdivisions):
        mids: dict[tuple[int, int], int] = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in mids:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mids[key] = len(verts) - 1
            return mids[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = nf
    v = np.array(verts) * radius
    if seed is not None:
        v *= 1 + np.random.default_rng(seed).uniform(-jitter, jitter, (len(v), 1))
    return v.astype(np.float32), np.array(faces, np.int32)


def box_particles(lo, hi, dx: float, seed: int = 0) -> np.ndarray:
    """Particles filling the box [lo, hi] at 8 per cell (spacing dx / 2)."""
    v, t = unit_cube_mesh()
    m = translate(*lo) @ scale(*np.subtract(hi, lo))
    return geometry.sample_mesh_volume(geometry.transform_points(m, v), t, dx / 2, seed)


def sphere_particles(center, radius: float, dx: float, seed: int = 0, spacing_div: float = 2.0) -> np.ndarray:
    v, t = icosphere(radius, 4)
    return geometry.sample_mesh_volume(v + np.asarray(center, np.float32), t, dx / spacing_div, seed)


def domain(lo=(0, 0, 0), hi=(1, 1, 1), res: int = 64, walls=None, wall_friction: float = 0.5) -> Domain:
    return Domain(tuple(lo), tuple(hi), res, dict(walls or ALL_WALLS), wall_friction)


def add(solver, positions, material_id: int = 0, emitter_id: int = 0, velocity=(0.0, 0.0, 0.0)) -> None:
    n = len(positions)
    solver.add_particles(positions, np.tile(np.asarray(velocity, np.float32), (n, 1)),
                         np.full(n, material_id, np.int32), np.full(n, emitter_id, np.int32))


def perturbed_state(solver_state: dict, seed: int, v_scale=0.3, c_scale=1.0, f_scale=0.05) -> dict:
    rng = np.random.default_rng(seed)
    s = {k: np.array(v) for k, v in solver_state.items()}
    n = len(s["x"])
    s["v"] = (s["v"] + rng.normal(0, v_scale, (n, 3))).astype(np.float32)
    s["C"] = rng.normal(0, c_scale, (n, 3, 3)).astype(np.float32)
    s["F"] = (np.eye(3) + rng.normal(0, f_scale, (n, 3, 3))).astype(np.float32)
    s["Jp"] = (1.0 + rng.normal(0, 0.02, n)).astype(np.float32)
    return s


def mix_scene(res: int = 128, seed: int = 0):
    """The mixed-materials workload: von Mises sphere r=0.12, Drucker-Prager column 0.15 x 0.4 x 0.15 (35 deg),
    snowball r=0.08 thrown at (3, 1, 0) m/s, one static seeded perturbed icosphere collider (5,120 triangles),
    all in a 1 m box at 8 particles per cell.

    Returns (domain, materials, particle groups [(positions, material, velocity)], collider (verts, tris, xf)).
    """
    d = domain(res=res)
    dx = d.dx
    mats = [MaterialParams("vm_sphere", "von_mises", 2e4, 0.45, 600.0, yield_stress=300.0),
            MaterialParams("dp_column", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=35.0),
            MaterialParams("snowball", "snow", 1.4e5, 0.2, 400.0, hardening=10.0, critical_compression=2.5e-2,
                           critical_stretch=7.5e-3, max_hardening=20.0)]
    groups = [(sphere_particles((0.25, 0.5, 0.3), 0.12, dx, seed=seed), 0, (0.0, 0.0, 0.0)),
              (box_particles((0.5, 0.425, 0.0), (0.65, 0.575, 0.4), dx, seed=seed + 1), 1, (0.0, 0.0, 0.0)),
              (sphere_particles((0.8, 0.3, 0.5), 0.08, dx, seed=seed + 2), 2, (3.0, 1.0, 0.0))]
    # snowball thrown at (3, 1, 0) m/s: place it on the -x side so it flies into the scene
    groups[2] = (groups[2][0] - np.array([0.6, 0.0, 0.0], np.float32), 2, (3.0, 1.0, 0.0))
    cv, ct = icosphere(1.0, 4, seed=seed + 3, jitter=0.03)
    xf = translate(0.75, 0.7, 0.1) @ scale(0.12)
    return d, mats, groups, (cv, ct, xf)


def lattice_box(lo, hi, spacing: float, rng) -> np.ndarray:
    """Particles on a lattice of the given spacing filling [lo, hi], each jittered by U(+-spacing / 4)."""
    axes = [np.arange(lo[a] + spacing / 2, hi[a], spacing, dtype=np.float64) for a in range(3)]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    g += rng.uniform(-0.25 * spacing, 0.25 * spacing, g.shape)
    return g.astype(np.float32)


BATCH_MODELS = ("elastic", "von_mises", "drucker_prager", "snow")


def batched_scenes(seed: int = 0, count: int = 64, n_lo: float = 1e4, n_hi: float = 2e6):
    """Independent scenes of the batched workload: particle counts log-uniform in [n_lo, n_hi], grids from 32^3
    to 192^3 matched to the count (a cube of material filling the same fraction of every grid, 8 per cell),
    one material per scene with the model uniform over the four and parameters uniform within the ranges of the
    jelly and mixed-materials workloads, a random initial velocity, and 0-2 static seeded perturbed icosphere
    colliders of 1,280, 5,120 or 20,480 triangles below the material.

    Returns [(domain, [material], positions, velocity, [(verts, tris, world matrix, friction)])].
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n_target = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        res = int(np.clip(round(32 * (n_target / 1e4) ** (1 / 3)), 32, 192))
        d = domain(res=res)
        side = min((n_target / 8) ** (1 / 3) / res, 0.6)
        lo = (0.5 - side / 2, 0.5 - side / 2, 0.25)
        hi = (0.5 + side / 2, 0.5 + side / 2, 0.25 + side)
        pos = lattice_box(lo, hi, d.dx / 2, rng)
        model = BATCH_MODELS[int(rng.integers(4))]
        mat = MaterialParams(f"batch{i}", model, float(rng.uniform(2e4, 3.5e5)), float(rng.uniform(0.2, 0.45)),
                             float(rng.uniform(400.0, 1600.0)), yield_stress=float(rng.uniform(300.0, 3000.0)),
                             friction_angle_deg=float(rng.uniform(30.0, 35.0)), hardening=10.0,
                             critical_compression=2.5e-2, critical_stretch=7.5e-3,
                             max_hardening=float(rng.uniform(5.0, 20.0)))
        vel = tuple(float(c) for c in rng.uniform(-1.0, 1.0, 3))
        cols = []
        for c in range(int(rng.integers(0, 3))):
            cv, ct = icosphere(1.0, int(rng.choice([3, 4, 5])), seed=seed * 1000 + i * 10 + c, jitter=0.03)
            r = float(rng.uniform(0.06, 0.12))
            xf = translate(float(rng.uniform(0.25, 0.75)), float(rng.uniform(0.25, 0.75)), r) @ scale(r)
            cols.append((cv, ct, xf, float(rng.uniform(0.0, 0.5))))
        out.append((d, [mat], pos, vel, cols))
    return out


def torus(major: float, minor: float, n_major: int, n_minor: int, seed: int | None = None, jitter: float = 0.0):
    """Closed torus around the z axis (2 * n_major * n_minor triangles, outward winding); with a seed every
    vertex's tube radius is scaled by 1 + U(-jitter, jitter)."""
    u = 2 * np.pi * np.arange(n_major) / n_major
    v = 2 * np.pi * np.arange(n_minor) / n_minor
    r = np.full((n_major, n_minor), minor)
    if seed is not None:
        r = r * (1 + np.random.default_rng(seed).uniform(-jitter, jitter, r.shape))
    cu, su, cv, sv = np.cos(u)[:, None], np.sin(u)[:, None], np.cos(v)[None, :], np.sin(v)[None, :]
    verts = np.stack([(major + r * cv) * cu, (major + r * cv) * su, r * sv], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    a = i * n_minor + j
    b = ((i + 1) % n_major) * n_minor + j
    c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
    d = i * n_minor + (j + 1) % n_minor
    tris = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return verts.astype(np.float32), tris.astype(np.int32)


def rot_z(deg: float) -> np.ndarray:
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    m = np.eye(4)
    m[:2, :2] = [[c, -s], [s, c]]
    return m


def pour_job_spec(seed: int, res: int = 96, frames: int = 12, fps: float = 24.0, side_range=(0.2, 0.4)):
    """A granular pour (the large inflow workload's distribution at a serving size): a Drucker-Prager pile
    (E 3.5e5, nu 0.3, 30 deg, rho 1600) of seeded size, a disc inflow r = 0.05 m at 2 m/s downward whose slab
    of one frame is added where no material is, and a seeded torus collider (2,048 triangles, friction 0.4)
    turning at 1 rev/s. Returns (domain, materials, setup(solver), before_frame(solver, k), frames, fps,
    max_particles, collider_triangles)."""
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    rng = np.random.default_rng(seed)
    d = domain(res=res)
    mat = MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)
    side = float(rng.uniform(*side_range))
    pile = lattice_box((0.5 - side / 2, 0.5 - side / 2, 0.0), (0.5 + side / 2, 0.5 + side / 2, side / 2), d.dx / 2,
                       rng)
    tv, tt = torus(0.18, 0.04, 64, 16, seed=seed, jitter=0.05)

    def pose(t):
        return translate(0.5, 0.5, 0.35) @ rot_z(360.0 * t) @ rot_x(90.0)

    def setup(s):
        s.add_particles(pile, np.zeros_like(pile), np.zeros(len(pile), np.int32), np.zeros(len(pile), np.int32))
        s.set_colliders([ColliderGeometry(MeshData(tv, tt), closed=True, friction=0.4)])

    def before_frame(s, k):
        s.set_collider_transforms(pose((k - 1) / fps)[None], pose(k / fps)[None])
        r = np.random.default_rng(seed * 1000 + k)
        slab = lattice_box((0.45, 0.45, 0.85), (0.55, 0.55, 0.85 + 2.0 / fps), d.dx / 2, r)
        slab = slab[np.hypot(slab[:, 0] - 0.5, slab[:, 1] - 0.5) <= 0.05]
        free = ~s.is_occupied(slab)
        if free.any():
            p = slab[free]
            s.add_particles(p, np.tile(np.float32([0.0, 0.0, -2.0]), (len(p), 1)), np.zeros(len(p), np.int32),
                            np.zeros(len(p), np.int32))

    slab_n = int(np.pi * 0.05 ** 2 * 2.0 / fps * 8 * res ** 3) + 1
    return d, [mat], setup, before_frame, frames, fps, len(pile) + frames * slab_n, len(tt)


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


def bake_scene(resolution: int = 16, frame_end: int = 4, emit_frames=(1, 3), substeps: int = 2,
               preset_name: str = "jelly", velocity=(0.0, 0.0, -1.0)):
    """A scene for the reference's bake runner (needs mpm_core): unit-cube domain, one closed cube inflow
    emitter "pour" above the floor (active over emit_frames, `substeps` emissions per frame), one open plane
    collider drifting along x by a cell per frame, jelly or another preset. Returns a SceneDescription."""
    from mpm_core.materials import load_preset
    from mpm_core.scene import Collider, Emitter, SceneDescription
    from mpm_core.scene import Domain as CoreDomain
    from mpm_core.scene import MeshData as CoreMesh

    n = frame_end
    dx = 1.0 / resolution
    cube_v, cube_t = unit_cube_mesh()
    emitter = Emitter(name="pour", kind="inflow", material=0, mesh=CoreMesh(cube_v, cube_t),
                      transforms=np.repeat((translate(0.35, 0.35, 0.55) @ scale(0.3, 0.3, 0.25))[None], n, 0),
                      velocity=tuple(velocity), frame_start=emit_frames[0], frame_end=emit_frames[1],
                      substeps=substeps)
    pv, pt = plane_mesh(0.8)
    floor = Collider(name="floor", mesh=CoreMesh(pv, pt),
                     transforms=np.stack([translate(0.5 + k * dx, 0.5, 0.1) for k in range(n)]), friction=0.5,
                     closed=False)
    return SceneDescription(domain=CoreDomain((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), resolution),
                            materials=[load_preset(preset_name).material], emitters=[emitter], colliders=[floor],
                            frame_start=1, frame_end=frame_end)


def cache_contents(cache_dir) -> dict:
    """{relative path: content} of a bake cache for comparisons: every frame and checkpoint archive as its
    members' raw bytes (the .npy payloads; zip member timestamps left out), cache.json as text. The progress
    file (timings) is left out."""
    import zipfile
    from pathlib import Path

    root = Path(cache_dir)
    out = {}
    for p in sorted(root.rglob("*")):
        rel = str(p.relative_to(root))
        if p.is_dir() or rel.startswith("scene") or rel in ("progress.json", "bake.lock"):
            continue
        if p.suffix == ".npz":
            with zipfile.ZipFile(p) as z:
                out[rel] = {name: z.read(name) for name in sorted(z.namelist())}
        else:
            out[rel] = p.read_bytes()
    return out

"""Seeded test scenes: meshes, particle boxes/spheres, matrices and the reference's material presets.

Particles are sampled with the oracle's restatement of the reference's volume sampler (pinned by the golden
fixtures), so the same seeds give the same particles as the reference's own test helpers.
"""

from __future__ import annotations

import json

import numpy as np
from _golden import GOLDEN, Domain, material_from_dict

from mpm_plugin_gb300.interface import MaterialParams
from mpm_plugin_gb300.workloads import (cylinder, lattice_box, plane_mesh, rot_x, rot_y, rot_z, scale,  # noqa: F401
                                        torus, translate)
from mpm_plugin_gb300.workloads import pour_job as pour_job_spec  # noqa: F401
from oracle import geometry

WALL_SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")
ALL_WALLS = {side: True for side in WALL_SIDES}

_PRESETS = json.loads(str(np.load(GOLDEN / "geometry.npz")["meta"]))["presets"]


def preset(name: str) -> MaterialParams:
    """Material parameters of the reference's built-in preset ``name`` (mpm_core/presets/*.toml)."""
    return material_from_dict(_PRESETS[name]["material"])


def preset_names() -> list[str]:
    return sorted(_PRESETS)


def unit_cube_mesh(centered: bool = False):
    """Closed cube with outward winding: [0,1]^3, or [-0.5,0.5]^3 when centered."""
    v = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32)
    if centered:
        v -= 0.5
    t = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                  [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]], np.int32)
    return v, t


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

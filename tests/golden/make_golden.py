"""Generate the golden fixtures in this folder by running the reference's own MLS-MPM code.

    python tests/golden/make_golden.py --reference PATH_TO_MPM_PLUGIN_CHECKOUT [--only NAME ...]

(or MPM_PLUGIN_REFERENCE=PATH in the environment instead of --reference)

The reference backend (``mpm_core/backends/warp/{solver,kernels,colliders}.py``) is imported from the
reference checkout and run unchanged on the CPU through ``warp_emu`` (a CPU emulator of the Warp API subset
it uses; warp-lang itself is not installable here). Its host-side helpers (``mpm_core.geometry``,
``mpm_core.bake._emission_times``, ``MaterialParams.lame``) are called directly. Each case is written as
``<name>.npz``: the inputs, the reference's outputs and a JSON ``meta`` string describing the scene.

Only this script reads the reference; the tests read the ``.npz`` files it wrote.
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
STATE_KEYS = ("x", "v", "C", "F", "Jp", "mat", "emitter")


def _install(reference: Path):
    sys.path.insert(0, str(HERE))
    import warp_emu

    sys.modules["warp"] = warp_emu
    sys.path.insert(0, str(reference / "src"))
    sys.path.insert(0, str(reference / "tests"))


def _domain_dict(d) -> dict:
    return {"min": list(d.min), "max": list(d.max), "resolution": d.resolution, "walls": dict(d.walls),
            "wall_friction": d.wall_friction}


def _perturb(state: dict, rng, v_scale=0.5, c_scale=2.0, f_scale=0.1) -> dict:
    n = len(state["x"])
    s = {k: np.array(v) for k, v in state.items()}
    s["v"] = (s["v"] + rng.normal(0, v_scale, (n, 3))).astype(np.float32)
    s["C"] = rng.normal(0, c_scale, (n, 3, 3)).astype(np.float32)
    s["F"] = (np.eye(3) + rng.normal(0, f_scale, (n, 3, 3))).astype(np.float32)
    s["Jp"] = (1.0 + rng.normal(0, 0.02, n)).astype(np.float32)
    return s


def run_case(name, domain, materials, particles, *, gravity=(0.0, 0.0, -9.81), ppc=8, colliders=(),
             transforms=None, perturb=None, action, seed=0, special=None):
    """particles: list of (positions, material_id, emitter_id, velocity(3,))."""
    from mpm_core.backends.warp.solver import WarpSolver
    from mpm_core.solver import ColliderGeometry

    t0 = time.time()
    solver = WarpSolver(domain=domain, materials=materials, gravity=gravity, particles_per_cell=ppc)
    for pos, mid, eid, vel in particles:
        n = len(pos)
        solver.add_particles(pos, np.tile(np.asarray(vel, np.float32), (n, 1)), np.full(n, mid, np.int32),
                             np.full(n, eid, np.int32))
    rng = np.random.default_rng(seed)
    state = solver.save_state()
    if perturb:
        state = _perturb(state, rng, **perturb)
    if special:
        state = special(state, rng)
    solver.load_state(state)
    cols = [ColliderGeometry(mesh, closed, friction) for mesh, closed, friction in colliders]
    solver.set_colliders(cols)
    if transforms is not None:
        solver.set_collider_transforms(*transforms)
    state_in = solver.save_state()

    out = {f"in_{k}": v for k, v in state_in.items()}
    meta = {"case": name, "domain": _domain_dict(domain), "materials": [m.to_dict() for m in materials],
            "gravity": list(gravity), "ppc": ppc,
            "colliders": [{"closed": bool(c), "friction": float(f)} for _, c, f in colliders],
            "action": action}
    for i, (mesh, _, _) in enumerate(colliders):
        out[f"col{i}_verts"] = mesh.verts
        out[f"col{i}_tris"] = mesh.tris
    if transforms is not None:
        out["xf_start"] = np.asarray(transforms[0], np.float32)
        out["xf_end"] = np.asarray(transforms[1], np.float32)

    kind = action["kind"]
    if kind == "substep":
        solver._frame_dt = action["frame_dt"]
        for k in range(action.get("count", 1)):
            solver._substep(action["dt"], action["s"][k] if isinstance(action["s"], list) else action["s"])
    elif kind == "advance":
        stats = []
        for frame_dt in action["frame_dts"]:
            st = solver.advance(frame_dt)
            stats.append([st.substeps, st.dt, st.removed])
        out["stats"] = np.array(stats, np.float64)
    elif kind == "occupied":
        out["points"] = np.asarray(action.pop("points"), np.float32)
        out["occupied"] = solver.is_occupied(out["points"])
    state_out = solver.save_state()
    out.update({f"out_{k}": v for k, v in state_out.items()})
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: {len(state_in['x'])} -> {len(state_out['x'])} particles, {time.time() - t0:.1f} s")


def solver_cases(only):
    from helpers import box_particles, icosphere, plane_mesh, scale, translate, unit_cube_mesh

    from mpm_core.materials import load_preset
    from mpm_core.scene import Domain, MeshData
    from mpm_core.geometry import transform_points

    def rot_y(deg):
        a = np.radians(deg)
        m = np.eye(4, dtype=np.float32)
        m[0, 0], m[0, 2], m[2, 0], m[2, 2] = np.cos(a), np.sin(a), -np.sin(a), np.cos(a)
        return m

    def rot_x(deg):
        a = np.radians(deg)
        m = np.eye(4, dtype=np.float32)
        m[1, 1], m[1, 2], m[2, 1], m[2, 2] = np.cos(a), -np.sin(a), np.sin(a), np.cos(a)
        return m

    P = {k: load_preset(k).material for k in ("jelly", "mashed_potato", "sand_dry", "snow_packed",
                                                 "whipped_cream", "rubber")}
    cases = {}

    d16 = Domain((0, 0, 0), (1, 1, 1), 16)
    cases["elastic_substep"] = lambda: run_case(
        "elastic_substep", d16, [P["jelly"]], [(box_particles((0.375,) * 3, (0.625,) * 3, d16.dx), 0, 0, (0, 0, 0))],
        perturb={"v_scale": 0.5, "c_scale": 2.0, "f_scale": 0.1}, seed=1,
        action={"kind": "substep", "dt": 2e-3, "s": 1.0, "frame_dt": 1 / 24})

    def degenerate(state, rng):
        F = state["F"]
        F[0] = np.eye(3)  # identical singular values
        F[1] = np.diag([1.2, 1.2, 0.9])  # two equal singular values
        F[2] = np.diag([1.1, 0.95, -0.9])  # inverted (det < 0)
        F[3] = np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])  # reflection
        F[4] = np.diag([1.5, 0.6, 0.8])  # strong stretch: yields / clamps
        F[5] = np.diag([0.999, 0.998, 0.997])  # compression: DP inside the cone
        F[6] = np.diag([1e-6, 1.0, 1.0])  # nearly singular: safe_log floor
        state["F"] = F
        return state

    mix_mats = [P["jelly"], P["mashed_potato"], P["sand_dry"], P["snow_packed"]]
    mix_parts = [(box_particles((0.25, 0.25, 0.25), (0.375, 0.375, 0.375), d16.dx, seed=i), i, i, (0, 0, 0))
                 for i in range(4)]
    for i, (p, *_rest) in enumerate(mix_parts):
        p += np.array([0.25 * (i % 2), 0.25 * (i // 2), 0.0], np.float32)
    cases["models_substep"] = lambda: run_case(
        "models_substep", d16, mix_mats, mix_parts, perturb={"f_scale": 0.25, "c_scale": 4.0},
        special=degenerate, action={"kind": "substep", "dt": 1e-3, "s": 1.0, "frame_dt": 1 / 24}, seed=2)
    cases["models_3substeps"] = lambda: run_case(
        "models_3substeps", d16, mix_mats, mix_parts, perturb={"f_scale": 0.25, "c_scale": 4.0},
        action={"kind": "substep", "dt": 1e-3, "s": [1 / 3, 2 / 3, 1.0], "count": 3, "frame_dt": 3e-3}, seed=3)

    # walls: friction, a non-unit placement, open sides and particles leaving through them
    dw = Domain((0.1, -0.2, 0.013), (0.6, 0.3, 0.5132), 16,
                walls={"x-": True, "x+": False, "y-": True, "y+": True, "z-": True, "z+": False},
                wall_friction=0.5)
    wp1 = box_particles((0.1, -0.2, 0.013), (0.2, -0.05, 0.09), dw.dx, seed=4)
    wp2 = box_particles((0.5, 0.15, 0.4), (0.6, 0.3, 0.5132), dw.dx, seed=5)
    cases["walls_substep"] = lambda: run_case(
        "walls_substep", dw, [P["whipped_cream"]], [(wp1, 0, 0, (-1.0, -0.5, -2.0)), (wp2, 0, 1, (3.0, 1.0, 4.0))],
        perturb={"v_scale": 0.2, "c_scale": 1.0, "f_scale": 0.02}, seed=6,
        action={"kind": "substep", "dt": 1e-3, "s": 1.0, "frame_dt": 1 / 24})
    cases["walls_advance"] = lambda: run_case(
        "walls_advance", dw, [P["whipped_cream"]], [(wp1, 0, 0, (-1.0, -0.5, -2.0)), (wp2, 0, 1, (6.0, 1.0, 8.0))],
        seed=7, action={"kind": "advance", "frame_dts": [1 / 240, 1 / 240]})

    # colliders
    cube = MeshData(*unit_cube_mesh(centered=True))
    box0 = translate(0.5, 0.5, 0.2) @ rot_y(10) @ scale(0.5, 0.4, 0.2)
    box1 = translate(0.52, 0.5, 0.21) @ rot_y(14) @ scale(0.5, 0.4, 0.2)
    cb = box_particles((0.35, 0.35, 0.2), (0.65, 0.6, 0.4), d16.dx, seed=8)
    cases["collider_box_substep"] = lambda: run_case(
        "collider_box_substep", d16, [P["sand_dry"]], [(cb, 0, 0, (0.0, 0.0, -1.0))], colliders=[(cube, True, 0.5)],
        transforms=(box0[None], box1[None]), perturb={"v_scale": 0.3, "c_scale": 1.0, "f_scale": 0.02}, seed=9,
        action={"kind": "substep", "dt": 1e-3, "s": 0.5, "frame_dt": 1 / 24})

    plane = MeshData(*plane_mesh(0.8))
    pl0 = translate(0.5, 0.5, 0.3) @ rot_y(12)
    pl1 = translate(0.5, 0.5, 0.31) @ rot_y(15)
    local = box_particles((-0.1, -0.1, -0.1), (0.1, 0.1, 0.1), d16.dx, seed=10)
    cp = transform_points(pl0, local)
    cases["collider_plane_substep"] = lambda: run_case(
        "collider_plane_substep", d16, [P["whipped_cream"]], [(cp, 0, 0, (0.2, 0.0, -1.5))],
        colliders=[(plane, False, 0.3)], transforms=(pl0[None], pl1[None]),
        perturb={"v_scale": 0.3, "c_scale": 1.0, "f_scale": 0.02}, seed=11,
        action={"kind": "substep", "dt": 1e-3, "s": 0.75, "frame_dt": 1 / 24})

    sph = MeshData(*icosphere(1.0, 2))
    b0 = translate(0.5, 0.5, 0.3) @ rot_x(0) @ scale(0.15)
    b1 = translate(0.5, 0.52, 0.3) @ rot_x(40) @ scale(0.15)
    sp = box_particles((0.3, 0.3, 0.1), (0.7, 0.7, 0.45), d16.dx, seed=12)
    cases["collider_sphere_substep"] = lambda: run_case(
        "collider_sphere_substep", d16, [P["snow_packed"], P["rubber"]],
        [(sp[: len(sp) // 2], 0, 0, (0.0, 0.0, 0.0)), (sp[len(sp) // 2:], 1, 1, (0.5, 0.0, 0.0))],
        colliders=[(sph, True, 0.0), (cube, True, 0.8)],
        transforms=(np.stack([b0, translate(0.5, 0.5, -0.05) @ scale(1.2, 1.2, 0.2)]),
                    np.stack([b1, translate(0.5, 0.5, -0.04) @ scale(1.2, 1.2, 0.2)])),
        perturb={"v_scale": 0.3, "c_scale": 1.0, "f_scale": 0.05}, seed=13,
        action={"kind": "substep", "dt": 1e-3, "s": 0.4, "frame_dt": 1 / 48})

    def nan_v(state, rng):
        state["v"][0] = np.nan
        return state

    cases["nan_advance"] = lambda: run_case(
        "nan_advance", d16, [P["jelly"]], [(box_particles((0.4, 0.4, 0.0), (0.6, 0.6, 0.125), d16.dx), 0, 0, (0, 0, 0))],
        special=nan_v, action={"kind": "advance", "frame_dts": [1 / 480]})

    cases["jelly_advance"] = lambda: run_case(
        "jelly_advance", d16, [P["jelly"]],
        [(box_particles((0.375, 0.375, 0.25), (0.625, 0.625, 0.5), d16.dx), 0, 0, (0, 0, 0))],
        perturb={"v_scale": 0.3, "c_scale": 0.5, "f_scale": 0.02}, seed=14,
        action={"kind": "advance", "frame_dts": [1 / 96]})

    q = np.random.default_rng(15).uniform(-0.05, 1.05, (200, 3)).astype(np.float32)
    q[:4] = [[0.5, 0.5, 0.1], [0.9, 0.9, 0.9], [0.4, 0.4, 0.0], [-0.3, 0.5, 0.5]]
    cases["occupied"] = lambda: run_case(
        "occupied", d16, [P["jelly"]], [(box_particles((0.4, 0.4, 0.0), (0.6, 0.6, 0.2), d16.dx), 0, 0, (0, 0, 0))],
        action={"kind": "occupied", "points": q})

    for name, fn in cases.items():
        if not only or name in only:
            fn()


def geometry_cases(only):
    """Host-side helpers on the path: pose decomposition/interpolation, volume sampling, emission times."""
    if only and "geometry" not in only:
        return
    from helpers import icosphere, unit_cube_mesh

    from mpm_core.bake import _emission_times
    from mpm_core.geometry import decompose_transform, interpolate_transform, sample_mesh_volume, transform_points
    from mpm_core.materials import list_presets, load_preset
    from mpm_core.scene import Domain, Emitter, MeshData, SceneDescription
    from mpm_core.backends.warp.solver import _dp_alpha

    rng = np.random.default_rng(20)
    mats = []
    for i in range(24):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        x, y, z, w = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        S = np.diag(rng.uniform(0.2, 2.0, 3))
        if i % 6 == 5:
            S[0, 0] = -S[0, 0]  # mirrored
        if i % 6 == 4:
            S = np.eye(3) * rng.uniform(0.5, 2)  # uniform scale
        m = np.eye(4)
        m[:3, :3] = R @ S
        m[:3, 3] = rng.normal(size=3)
        mats.append(m.astype(np.float32))
    mats = np.stack(mats)
    t, q, S = zip(*(decompose_transform(m) for m in mats))
    svals = np.array([0.0, 0.25, 0.5, 0.8, 1.0])
    interp = np.stack([[interpolate_transform(mats[i], mats[i + 1], s) for s in svals] for i in range(0, 24, 2)])

    cube_v, cube_t = unit_cube_mesh()
    sph_v, sph_t = icosphere(0.13, 3)
    samples = {}
    samp_meta = []
    for k, (v, t_, spacing, seed, xf) in enumerate([
        (cube_v, cube_t, 1 / 64, 0, np.array([[0.25, 0, 0, 0.375], [0, 0.25, 0, 0.475], [0, 0, 0.25, 0.375],
                                              [0, 0, 0, 1]])),
        (cube_v, cube_t, 1 / 48, [3, 7, 1, 2, 4], np.diag([0.1, 0.3, 0.2, 1.0])),
        (sph_v, sph_t, 1 / 64, 5, np.eye(4)),
        (sph_v, sph_t, 1 / 90, [0, 12, 0, 1, 4], np.eye(4)),
    ]):
        wv = transform_points(np.asarray(xf, np.float32), v) + (np.float32(0.5) if k >= 2 else np.float32(0))
        pts = sample_mesh_volume(wv, t_, spacing, seed)
        samples[f"sample{k}_verts"] = wv
        samples[f"sample{k}_tris"] = t_
        samples[f"sample{k}_points"] = pts
        samp_meta.append({"spacing": spacing, "seed": seed})

    def emit_scene():
        cube = MeshData(cube_v, cube_t)
        xf = np.repeat(np.eye(4, dtype=np.float32)[None], 12, 0)
        return SceneDescription(
            domain=Domain((0, 0, 0), (1, 1, 1), 16), materials=[load_preset("jelly").material],
            emitters=[Emitter("a", "inflow", 0, cube, xf, frame_start=3, frame_end=8, substeps=4),
                      Emitter("b", "inflow", 0, cube, xf, frame_start=2, frame_end=10, substeps=3),
                      Emitter("c", "fill", 0, cube, xf)],
            colliders=[], frame_start=1, frame_end=12)

    sc = emit_scene()
    times = {f: [[str(s), e] for s, e in _emission_times(sc, f)] for f in range(1, 13)}

    presets = {}
    for pid in list_presets():
        m = load_preset(pid).material
        mu, lam = m.lame()
        presets[pid] = {"material": m.to_dict(), "mu": mu, "lam": lam, "alpha": _dp_alpha(m.friction_angle_deg)}

    domains = []
    for dmin, dmax, res in [((0, 0, 0), (1, 1, 1), 64), ((-0.5, -0.2, 0.0), (0.5, 0.05, 0.5), 64),
                            ((0.1, -0.2, 0.013), (0.6, 0.3, 0.5132), 16), ((0, 0, 1.0359), (1, 1, 2.0359), 64),
                            ((0, 0, 0), (1, 1, 1), 128), ((0, 0, 0), (1, 1, 1), 256), ((0, 0, 0.1326), (1, 1, 1.1326), 64)]:
        d = Domain(dmin, dmax, res)
        domains.append({"min": list(d.min), "max": list(d.max), "resolution": res, "dx": d.dx,
                        "grid_shape": list(d.grid_shape)})

    meta = {"case": "geometry", "svals": svals.tolist(), "samples": samp_meta, "emission_times": times,
            "presets": presets, "domains": domains}
    np.savez_compressed(HERE / "geometry.npz", mats=mats, t=np.stack(t), q=np.stack(q), S=np.stack(S),
                        interp=interp, meta=np.array(json.dumps(meta)), **samples)
    print("geometry: written")


def surface_cases(only):
    """The surfacer's field stage (mpm_surface/field.py): the reference's unchanged surface_particles on a
    seeded particle blob, with its splat, normalize and sample_velocity kernels run by the emulator. Warp's
    MarchingCubes (not in the reference's sources) is replaced by a stand-in that keeps the density field it
    is given and hands back a set of sample points, so the reference's own code samples its velocity field at
    them (field.py:131-136)."""
    if only and "surface_field" not in only:
        return
    import warp as wp
    from mpm_surface import field
    from mpm_surface.settings import SurfaceSettings

    rng = np.random.default_rng(41)
    spacing = 0.01
    g = (np.stack(np.meshgrid(*[np.arange(8)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * spacing
    c = g.mean(0)
    pts = g[np.linalg.norm(g - c, axis=1) < 3.6 * spacing]
    pts = (pts + rng.uniform(-0.25, 0.25, pts.shape) * spacing + np.array([0.3, 0.5, 0.2])).astype(np.float32)
    vel = (np.cross(np.array([0.0, 0.0, 2.0]), pts - pts.mean(0)) + rng.normal(0, 0.05, pts.shape)).astype(np.float32)
    captured = {}

    class SampleOnly:  # in place of wp.MarchingCubes
        def __init__(self, nx, ny, nz, device=None):
            self.dims = (nx, ny, nz)
            r = np.random.default_rng(42)
            self.verts = wp.array(r.uniform(0.0, 1.0, (400, 3)) * (np.array(self.dims) - 1), dtype=wp.vec3)
            self.indices = wp.array(np.zeros(3, np.int32), dtype=int)

        def surface(self, density, iso):
            captured["density"] = density.numpy()
            captured["verts"] = self.verts.numpy()

    wp.MarchingCubes = SampleOnly
    out = {}
    for name, st in (("d1_s2", SurfaceSettings(detail=1.0, smoothing=2.0, iso=0.35)),
                     ("d15_s15", SurfaceSettings(detail=1.5, smoothing=1.5, iso=0.5))):
        mesh = field.surface_particles(pts, vel, spacing, st, device="cpu", max_bytes=1 << 40)
        out[f"{name}_density"] = captured["density"]   # normalised density field (field.py:123)
        out[f"{name}_sample_grid"] = captured["verts"]  # sample points, grid index units
        out[f"{name}_sample_world"] = mesh.verts        # the same points in world space (field.py:139)
        out[f"{name}_sample_vel"] = mesh.vel            # velocity field sampled there (field.py:135-136)
        out[f"{name}_settings"] = np.array([st.detail, st.smoothing, st.iso])
    np.savez_compressed(HERE / "surface_field.npz", positions=pts, velocities=vel, spacing=np.float64(spacing),
                        meta=np.array(json.dumps({"case": "surface_field", "cases": ["d1_s2", "d15_s15"]})), **out)
    print("surface_field: written")


def main() -> None:
    ap = argparse.ArgumentParser()
    env = os.environ.get("MPM_PLUGIN_REFERENCE")
    ap.add_argument("--reference", type=Path, default=Path(env) if env else None,
                    required=env is None, help="checkout of jonatanhedborg/mpm_plugin (or $MPM_PLUGIN_REFERENCE)")
    ap.add_argument("--only", nargs="*", default=[])
    args = ap.parse_args()
    _install(args.reference)
    geometry_cases(set(args.only))
    solver_cases(set(args.only))
    surface_cases(set(args.only))


if __name__ == "__main__":
    main()

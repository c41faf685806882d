"""Collider contact at the parity bar: one substep with material in the colliders' contact band, GPU (through
the C-ABI) against the FP32 oracle, within 1e-5 relative.

Three scenes, each with thousands of particles whose stencil nodes lie inside the 1-dx band of a mesh (the
grid-node contact of colliders.py:77-117) and particles inside the mesh that the projection
(colliders.py:120-148) pushes out:

* rest: the mixed-materials workload (304k particles, 128^3) with its seeded perturbed 5,120-triangle
  icosphere moved under the Drucker-Prager column, the column material around it;
* box: a closed cube collider translating and turning during the frame (poses interpolated at the substep's
  fraction s, colliders.py:30-37, and its velocity from them, colliders.py:68-74), granular material around it;
* torus: the large pour's seeded 20,480-triangle torus turning at 1 rev/s (per-frame start and end
  transforms, warp/solver.py:154-172) half buried in a Drucker-Prager pile.

The error is measured norm-wise per array over all particles and, separately, over the particles near the
surface only, so the contact region is not diluted by the free material. C (a near-cancelling sum) is
measured against the velocity-gradient scale |v| / dx. Each scene also runs without its collider, to show
that contact changes the result by far more than the tolerance.
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import (add, box_particles, domain, icosphere, lattice_box, mix_scene, perturbed_state, rot_x, rot_z,
                    scale, torus, translate, unit_cube_mesh)

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _sphere_dist(x, center, radius):
    return np.linalg.norm(x - np.asarray(center, np.float32), axis=1) - radius


def _box_dist(x, center, half):
    q = np.abs(x - np.asarray(center, np.float32)) - half
    return np.linalg.norm(np.maximum(q, 0.0), axis=1) + np.minimum(q.max(1), 0.0)


def _torus_dist(x, xf, major, minor):
    inv = np.linalg.inv(np.asarray(xf, np.float64))
    p = x.astype(np.float64) @ inv[:3, :3].T + inv[:3, 3]
    return np.hypot(np.hypot(p[:, 0], p[:, 1]) - major, p[:, 2]) - minor


def _scene(name):
    """(domain, materials, [(positions, material, velocity)], [(verts, tris, closed, friction)], start, end,
    s, dt, surface distance of a point) for one contact scene."""
    from mpm_plugin_gb300.interface import MaterialParams

    if name == "rest":
        d, mats, groups, (cv, ct, _) = mix_scene(res=128)
        center, r = (0.575, 0.5, 0.13), 0.12
        xf = translate(*center) @ scale(r)
        # the column's material around the sphere; particles deeper than 0.3 dx inside it are left out, the
        # shallower ones stay for the projection
        col = groups[1][0]
        keep = _sphere_dist(col, center, r * 1.03) > -0.3 * d.dx - 0.06 * r
        groups[1] = (col[keep], 1, (0.0, 0.0, 0.0))
        cols = [(cv, ct, True, 0.5)]
        return d, mats, groups, cols, xf[None], xf[None], 1.0, 5e-5, lambda x: _sphere_dist(x, center, r)
    if name == "box":
        d = domain(res=64)
        mats = [MaterialParams("sand", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0),
                MaterialParams("jelly", "elastic", 1e5, 0.3, 1000.0)]
        cv, ct = unit_cube_mesh(centered=True)
        start = translate(0.5, 0.5, 0.3) @ rot_z(10.0) @ scale(0.2)
        end = translate(0.55, 0.48, 0.3) @ rot_z(25.0) @ scale(0.2)
        rng = np.random.default_rng(21)
        pos = lattice_box((0.3, 0.3, 0.12), (0.72, 0.7, 0.5), d.dx / 2, rng)
        mid = translate(0.525, 0.49, 0.3) @ rot_z(17.5)
        local = (pos.astype(np.float64) - mid[:3, 3]) @ mid[:3, :3]
        keep = _box_dist(local, (0.0, 0.0, 0.0), 0.1) > -0.4 * d.dx
        pos = pos[keep]
        half = len(pos) // 2
        groups = [(pos[:half], 0, (0.0, 0.0, -0.5)), (pos[half:], 1, (0.2, 0.0, -0.5))]
        cols = [(cv, ct, True, 0.3)]
        return (d, mats, groups, cols, start[None].astype(np.float32), end[None].astype(np.float32), 0.5, 1e-4,
                lambda x: _box_dist((x.astype(np.float64) - mid[:3, 3]) @ mid[:3, :3], (0.0, 0.0, 0.0), 0.1))
    assert name == "torus"
    d = domain(res=128)
    mats = [MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)]
    tv, tt = torus(1.0, 0.22, 128, 80, seed=7, jitter=0.03)

    def rigid(t):  # the turning pose without the mesh's scale, for distances in world units
        return translate(0.5, 0.5, 0.22) @ rot_z(360.0 * t) @ rot_x(90.0)

    t0 = 5 / 24
    start, end = rigid(t0) @ scale(0.18), rigid(t0 + 1 / 24) @ scale(0.18)
    rng = np.random.default_rng(33)
    pile = lattice_box((0.25, 0.25, 0.0), (0.75, 0.75, 0.24), d.dx / 2, rng)
    s = 0.75
    now = rigid(t0 + s / 24)
    keep = _torus_dist(pile, now, 0.18, 0.18 * 0.22 * 1.03) > -0.4 * d.dx
    groups = [(pile[keep], 0, (0.0, 0.0, -1.0))]
    cols = [(tv, tt, True, 0.4)]
    return (d, mats, groups, cols, start[None].astype(np.float32), end[None].astype(np.float32), s, 5e-5,
            lambda x: _torus_dist(x, now, 0.18, 0.18 * 0.22))


def _run(name, with_collider=True, oracle=True):
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver
    from oracle.oracle import OracleSolver

    d, mats, groups, cols, start, end, s, dt, dist = _scene(name)
    g = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device="cuda:0")
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=8)
    for pos, m, vel in groups:
        add(g, pos, m, m, vel)
    state = perturbed_state(g.save_state(), seed=17, v_scale=0.2, c_scale=0.5, f_scale=0.02)
    for solver in (g, o):
        solver.load_state(state)
    if with_collider:
        g.set_colliders([ColliderGeometry(MeshData(v, t), c, f) for v, t, c, f in cols])
        g.set_collider_transforms(start, end)
        o.set_colliders(cols)
        o.set_collider_transforms(start, end)
    g.substep(dt, s, 1 / 24)
    out = g.save_state()
    g.close()
    if not oracle:
        return d, state, out, None, dist
    o.frame_dt = 1 / 24
    o.substep(dt, s)
    return d, state, out, o.save_state(), dist


def _errors(out, ref, dx, sel=None):
    sel = np.ones(len(ref["x"]), bool) if sel is None else sel
    gnorm = float(np.linalg.norm(ref["v"][sel]) / dx)
    return {k: rel_err(out[k][sel], ref[k][sel], floor=gnorm if k == "C" else 0.0)
            for k in ("x", "v", "C", "F", "Jp")}


@pytest.mark.parametrize("name", ["rest", "box", "torus"])
def test_contact_substep_matches_oracle(name):
    d, state, out, ref, dist = _run(name)
    near = np.abs(dist(state["x"])) < 2.0 * d.dx
    inside = dist(state["x"]) < 0.0
    assert near.sum() > 1000 and inside.sum() > 50, (near.sum(), inside.sum())
    every, contact = _errors(out, ref, d.dx), _errors(out, ref, d.dx, near)
    print(name, len(ref["x"]), "near", int(near.sum()), "inside", int(inside.sum()),
          "all", {k: f"{e:.1e}" for k, e in every.items()}, "near", {k: f"{e:.1e}" for k, e in contact.items()})
    for k in every:
        assert every[k] <= TOL, ("all", k, every[k])
        assert contact[k] <= TOL, ("near", k, contact[k])
    np.testing.assert_array_equal(np.isfinite(out["x"]), np.isfinite(ref["x"]))


@pytest.mark.parametrize("name", ["rest", "torus"])
def test_contact_changes_the_result(name):
    """Without the collider the same substep differs near the surface by orders of magnitude more than the
    tolerance: the comparison above is a comparison of contact, not of free flight."""
    d, state, out, _, dist = _run(name, with_collider=False, oracle=False)
    _, _, out_c, _, _ = _run(name, oracle=False)
    near = np.abs(dist(state["x"])) < 2.0 * d.dx
    inside = dist(state["x"]) < 0.0
    e_v, e_x = rel_err(out_c["v"][near], out["v"][near]), rel_err(out_c["x"][inside], out["x"][inside])
    print(name, "collider vs none: v near", f"{e_v:.1e}", "x inside", f"{e_x:.1e}")
    assert e_v > 1e3 * TOL and e_x > 10 * TOL  # contact and projection both acted


def test_collider_poses_are_reused_only_while_their_inputs_hold():
    """Explicit substeps at the same substep fraction with unchanged transforms reuse the poses already on the
    device (no pose launch); a new fraction, new transforms or a multi-substep call compute them again, and
    every pose read back equals the one a fresh solver computes for the same inputs, bit for bit."""
    from scenes import preset

    from mpm_plugin_gb300 import _abi, create
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    d = domain(res=32)

    def box(x, ang):
        return translate(x, 0.5, 0.3) @ rot_z(ang) @ scale(0.2, 0.2, 0.1)

    def make(xf0, xf1):
        s = create(domain=d, materials=[preset("sand_dry")], gravity=(0.0, 0.0, -9.81), device="cuda:0")
        s.set_option(_abi.OPT_SORT_INTERVAL, 0)
        add(s, box_particles((0.3, 0.3, 0.4), (0.7, 0.7, 0.5), d.dx))
        s.set_colliders([ColliderGeometry(MeshData(*unit_cube_mesh(centered=True)), closed=True, friction=0.5)])
        s.set_collider_transforms(xf0[None], xf1[None])
        return s

    def fresh_pose(xf0, xf1, sfrac):
        f = make(xf0, xf1)
        f.substep(1e-4, sfrac, 1 / 24)
        return f.read_collider_pose(0)

    def same(a, b):
        return all(np.array_equal(x, y) for x, y in zip(a, b))

    a0, a1 = box(0.45, 0.0), box(0.55, 20.0)
    s = make(a0, a1)
    s.substep(1e-4, 0.5, 1 / 24)  # builds the voxel grid and the graph
    n0 = s.launch_count()
    s.substep(1e-4, 0.5, 1 / 24)
    n_same = s.launch_count() - n0
    assert same(s.read_collider_pose(0), fresh_pose(a0, a1, 0.5))
    n0 = s.launch_count()
    s.substep(1e-4, 0.75, 1 / 24)
    assert s.launch_count() - n0 == n_same + 1  # the pose launch
    p75 = s.read_collider_pose(0)
    assert same(p75, fresh_pose(a0, a1, 0.75)) and not np.array_equal(p75[0], fresh_pose(a0, a1, 0.5)[0])
    b0, b1 = box(0.5, 10.0), box(0.6, 30.0)
    s.set_collider_transforms(b0[None], b1[None])
    n0 = s.launch_count()
    s.substep(1e-4, 0.75, 1 / 24)
    assert s.launch_count() - n0 == n_same + 1
    assert same(s.read_collider_pose(0), fresh_pose(b0, b1, 0.75))
    s.run_substeps(1e-4, 4, 1 / 24)  # poses of four substeps ending at s = 1
    s.substep(1e-4, 0.75, 1 / 24)  # recomputed after the multi-substep call
    assert same(s.read_collider_pose(0), fresh_pose(b0, b1, 0.75))

"""Parity of the sm_103a backend (through the C-ABI) with the reference and with the C oracle.

1. The golden fixtures (the reference's own kernels run on seeded scenes) replayed through Gb300Solver.
2. Larger seeded scenes against the FP32 oracle after one substep (x, v, C, F, Jp within 1e-5 relative,
   norm-wise per array; C, a near-cancelling sum, relative to the norm of the velocity gradient).
3. Conservation after 100 substeps (total mass, momentum, centre of mass, kinetic energy within 1e-4).
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import SOLVER_CASES, Case, rel_err
from scenes import add, box_particles, domain, mix_scene, perturbed_state, preset

pytestmark = pytest.mark.gpu

# Tolerance against the reference fixtures, the same for every fixture, colliders and multi-substep runs
# included: float atomics make the P2G sum order differ, and FMA contraction changes last-bit rounding, both
# at the 1e-7 level. C is measured against the velocity-gradient scale |v| / dx.
TOL = {"x": 1e-5, "v": 1e-5, "C": 1e-5, "F": 1e-5, "Jp": 1e-5}


def gpu_solver(domain_, materials, gravity=(0.0, 0.0, -9.81), ppc=8):
    from mpm_plugin_gb300.solver import Gb300Solver

    return Gb300Solver(domain_, materials, gravity, ppc, device="cuda:0")


def run_case_gpu(case: Case):
    s = gpu_solver(case.domain, case.materials, case.gravity, case.ppc)
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    s.load_state(case.state("in"))
    s.set_colliders([ColliderGeometry(MeshData(v, t), c, f) for v, t, c, f in case.colliders()])
    if case.transforms() is not None:
        s.set_collider_transforms(*case.transforms())
    a, extra = case.action, {}
    if a["kind"] == "substep":
        for k in range(a.get("count", 1)):
            s.substep(a["dt"], a["s"][k] if isinstance(a["s"], list) else a["s"], a["frame_dt"])
    elif a["kind"] == "advance":
        extra["stats"] = np.array([[st.substeps, st.dt, st.removed] for st in (s.advance(f) for f in a["frame_dts"])])
    elif a["kind"] == "occupied":
        extra["occupied"] = s.is_occupied(case.z["points"])
    return s.save_state(), extra


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_matches_reference_fixture(name):
    case = Case(name)
    out, extra = run_case_gpu(case)
    ref = case.state("out")
    assert len(out["x"]) == len(ref["x"])
    np.testing.assert_array_equal(out["mat"], ref["mat"])
    np.testing.assert_array_equal(out["emitter"], ref["emitter"])
    for k in ("x", "v"):
        np.testing.assert_array_equal(np.isfinite(out[k]), np.isfinite(ref[k]))
    gnorm = float(np.linalg.norm(ref["v"][np.isfinite(ref["v"]).all(1)]) / case.domain.dx)
    errs = {k: rel_err(out[k], ref[k], floor=gnorm if k == "C" else 0.0) for k in TOL}
    print(name, len(ref["x"]), {k: f"{e:.2e}" for k, e in errs.items()})
    for k, t in TOL.items():
        assert errs[k] <= t, (k, errs[k])
    if "stats" in extra:
        np.testing.assert_allclose(extra["stats"], case.z["stats"], rtol=1e-12)
    if "occupied" in extra:
        np.testing.assert_array_equal(extra["occupied"], case.z["occupied"])


def _oracle(domain_, materials, gravity=(0.0, 0.0, -9.81), precision="f32"):
    from oracle.oracle import OracleSolver

    return OracleSolver(domain_, materials, gravity, 8, precision=precision, threads=4)


def _velocity_gradient_norm(state, dx):
    return float(np.linalg.norm(state["v"]) / dx)


@pytest.mark.parametrize("scene", ["jelly64", "models32", "mix128_collider"])
def test_one_substep_matches_oracle(scene):
    """x, v, C, F, Jp after one substep within 1e-5 relative of the FP32 oracle."""
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    col = None
    if scene == "jelly64":
        d = domain(res=64)
        mats = [preset("jelly")]
        groups = [(box_particles((0.375, 0.475, 0.375), (0.625, 0.725, 0.625), d.dx, seed=0), 0, (0, 0, 0))]
        dt = 1e-4
    elif scene == "models32":
        d = domain(res=32)
        mats = [preset("jelly"), preset("mashed_potato"), preset("sand_dry"), preset("snow_packed")]
        groups = [(box_particles((0.1 + 0.2 * i, 0.3, 0.05), (0.25 + 0.2 * i, 0.6, 0.4), d.dx, seed=i), i, (0, 0, 0))
                  for i in range(4)]
        dt = 2e-4
    else:
        d, mats, groups, col = mix_scene(res=128)
        dt = 5e-5
    g = gpu_solver(d, mats)
    o = _oracle(d, mats)
    for pos, m, vel in groups:
        add(g, pos, m, m, vel)
        add(o, pos, m, m, vel)
    state = perturbed_state(g.save_state(), seed=11)
    g.load_state(state)
    o.load_state(state)
    if col is not None:
        cv, ct, xf = col
        g.set_colliders([ColliderGeometry(MeshData(cv, ct), True, 0.5)])
        g.set_collider_transforms(xf[None], xf[None])
        o.set_colliders([(cv, ct, True, 0.5)])
        o.set_collider_transforms(xf[None], xf[None])
    g.substep(dt, 1.0, 1 / 24)
    o.frame_dt = 1 / 24
    o.substep(dt, 1.0)
    out, ref = g.save_state(), o.save_state()
    gnorm = _velocity_gradient_norm(ref, d.dx)
    errs = {"x": rel_err(out["x"], ref["x"]), "v": rel_err(out["v"], ref["v"]),
            "C": rel_err(out["C"], ref["C"], floor=gnorm), "F": rel_err(out["F"], ref["F"]),
            "Jp": rel_err(out["Jp"], ref["Jp"])}
    print(scene, len(out["x"]), {k: f"{e:.2e}" for k, e in errs.items()}, "fp64 lanes", g.fp64_lanes())
    for k, e in errs.items():
        assert e <= 1e-5, (k, e)


@pytest.mark.parametrize("mode", [1, 2])
def test_fp64_clamp_is_closer_to_the_fp64_oracle(mode):
    """Sand (Drucker-Prager) and snow particles with the return mapping redone in FP64 (MPM_OPT_FP64_CLAMP):
    mode 1 redoes the lanes whose FP32 decision was marginal, mode 2 every lane whose clamp was active. One
    substep stays within 1e-5 of the FP32 oracle, and F, Jp and x are no further from the FP64 oracle than the
    FP32 build's; mode 1 redoes a small share of what mode 2 redoes."""
    from mpm_plugin_gb300 import _abi

    d = domain(res=32)
    mats = [preset("sand_dry"), preset("snow_packed")]
    groups = [(box_particles((0.1 + 0.4 * i, 0.3, 0.05), (0.45 + 0.4 * i, 0.6, 0.4), d.dx, seed=i), i, (0, 0, 0))
              for i in range(2)]
    gs = [gpu_solver(d, mats), gpu_solver(d, mats)]
    gs[1].set_option(_abi.OPT_FP64_CLAMP, mode)
    o32, o64 = _oracle(d, mats), _oracle(d, mats, precision="f64")
    for pos, m, vel in groups:
        add(gs[0], pos, m, m, vel)
    state = perturbed_state(gs[0].save_state(), seed=5)
    for s in (*gs, o32, o64):
        s.load_state(state)
    for s in gs:
        s.substep(2e-4, 1.0, 1 / 24)
    for o in (o32, o64):
        o.frame_dt = 1 / 24
        o.substep(2e-4, 1.0)
    plain, redo = gs[0].save_state(), gs[1].save_state()
    r32, r64 = o32.save_state(), o64.save_state()
    snow_clamped = (r64["mat"] == 1) & (r64["Jp"] != state["Jp"])  # snow's Jp changes only at the clamp
    assert snow_clamped.sum() > 100
    for k in ("x", "v", "F", "Jp"):
        assert rel_err(redo[k], r32[k]) <= 1e-5, k
    e_plain = {k: rel_err(plain[k], r64[k]) for k in ("x", "F", "Jp")}
    e_redo = {k: rel_err(redo[k], r64[k]) for k in ("x", "F", "Jp")}
    lanes = gs[1].fp64_redo_lanes()
    print(mode, lanes, "of", len(state["x"]), {k: f"{e_plain[k]:.2e} -> {e_redo[k]:.2e}" for k in e_plain})
    for k in e_plain:
        assert e_redo[k] <= 1.05 * e_plain[k] + 1e-9, (k, e_plain[k], e_redo[k])
    assert gs[0].fp64_redo_lanes() == 0
    if mode == 2:
        assert lanes >= snow_clamped.sum()
    else:
        assert lanes < 0.1 * len(state["x"])


def _invariants(s: dict, pmass: np.ndarray) -> dict:
    x, v = s["x"].astype(np.float64), s["v"].astype(np.float64)
    m = pmass.astype(np.float64)
    M = m.sum()
    return {"mass": M, "momentum": (m[:, None] * v).sum(0), "com": (m[:, None] * x).sum(0) / M,
            "ke": 0.5 * (m * (v * v).sum(1)).sum()}


def test_conservation_100_substeps_matches_oracle():
    d = domain(res=32)
    mats = [preset("jelly"), preset("sand_dry"), preset("snow_packed")]
    groups = [(box_particles((0.2, 0.3, 0.1), (0.4, 0.6, 0.4), d.dx, seed=1), 0, (1.0, 0.0, 0.0)),
              (box_particles((0.5, 0.3, 0.0), (0.7, 0.6, 0.3), d.dx, seed=2), 1, (0.0, 0.0, 0.0)),
              (box_particles((0.75, 0.4, 0.3), (0.9, 0.55, 0.45), d.dx, seed=3), 2, (-2.0, 0.0, 0.0))]
    g = gpu_solver(d, mats)
    o = _oracle(d, mats)
    for pos, m, vel in groups:
        add(g, pos, m, m, vel)
        add(o, pos, m, m, vel)
    for _ in range(100):
        g.substep(2e-4, 1.0, 1 / 24)
        o.substep(2e-4, 1.0)
    out, ref = g.save_state(), o.save_state()
    dx = d.dx
    pm = np.array([np.float32(m.density) * np.float32(dx ** 3 / 8) for m in mats], np.float32)[ref["mat"]]
    a, b = _invariants(out, pm), _invariants(ref, pm)
    print({k: (a[k], b[k]) for k in a})
    assert abs(a["mass"] - b["mass"]) <= 1e-4 * b["mass"]
    pscale = np.linalg.norm(b["momentum"]) + 1e-12
    assert np.linalg.norm(a["momentum"] - b["momentum"]) <= 1e-4 * pscale
    assert np.linalg.norm(a["com"] - b["com"]) <= 1e-4 * np.linalg.norm(b["com"])
    assert abs(a["ke"] - b["ke"]) <= 1e-4 * b["ke"]


def test_state_roundtrip_and_order():
    d = domain(res=32)
    g = gpu_solver(d, [preset("jelly")])
    pos = box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx)
    add(g, pos)
    s = g.save_state()
    np.testing.assert_array_equal(s["x"], pos)
    np.testing.assert_array_equal(s["F"], np.tile(np.eye(3, dtype=np.float32), (len(pos), 1, 1)))
    np.testing.assert_array_equal(s["Jp"], np.ones(len(pos), np.float32))
    p2 = perturbed_state(s, 3)
    g.load_state(p2)
    s2 = g.save_state()
    for k in s2:
        np.testing.assert_array_equal(s2[k], p2[k])


def test_frame_reads_share_one_state_read():
    """frame_reads (the bake entry point's solvers): get_particles reads the whole state and the save_state
    right after it returns that read; any advance in between makes save_state read afresh."""
    from mpm_plugin_gb300.solver import Gb300Solver

    d = domain(res=32)
    pos = box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx)
    a = Gb300Solver(d, [preset("jelly")], (0.0, 0.0, -9.81), 8, device="cuda:0", frame_reads=True)
    b = gpu_solver(d, [preset("jelly")])
    for s in (a, b):
        add(s, pos)
        s.advance(1 / 96)
    pa, pb = a.get_particles(), b.get_particles()
    fresh = a._save_state()
    for u, w, k in ((pa.positions, pb.positions, "x"), (pa.velocities, pb.velocities, "v"),
                    (pa.material_ids, pb.material_ids, "mat"), (pa.emitter_ids, pb.emitter_ids, "emitter")):
        assert u.dtype == w.dtype and u.shape == w.shape
        np.testing.assert_array_equal(u, fresh[k])
    sa = a.save_state()
    assert sa["x"] is pa.positions  # the same read
    for k in fresh:
        np.testing.assert_array_equal(sa[k], fresh[k])
    a.get_particles()
    a.advance(1 / 96)
    sa = a.save_state()
    assert np.abs(sa["x"] - pa.positions).max() > 0  # not the kept read
    fresh = a._save_state()
    for k in fresh:
        np.testing.assert_array_equal(sa[k], fresh[k])


@pytest.mark.parametrize("res", [64, 160])
def test_reorder_keeps_every_particle(res):
    """The reorder by grid node after every substep (counting sort over all grid nodes, 1,158 scan tiles at
    resolution 160) is a permutation: with dt = 0 positions and the other per-particle fields come back
    unchanged and in insertion order, NaN particles (sorted under the key past the last node) included.
    The first substep clamps the particles above the domain to the wall; the state is taken after it."""
    from mpm_plugin_gb300 import _abi

    d = domain(res=res)
    g = gpu_solver(d, [preset("jelly"), preset("sand_dry")])
    pos = box_particles((0.3, 0.3, 0.2), (0.7, 0.7, 0.5), d.dx, seed=4)
    mat = (np.arange(len(pos)) % 2).astype(np.int32)
    pos[::1000] = np.nan
    pos[500::1000] = (0.5, 0.5, 3.0)  # above the grid: its stencil leaves the padded grid
    g.add_particles(pos, np.zeros_like(pos), mat, np.arange(len(pos)) % 7)
    g.set_option(_abi.OPT_SORT_INTERVAL, 1)
    g.substep(0.0, 1.0, 1 / 24)
    s0 = g.save_state()
    assert np.isnan(s0["x"][::1000]).all()
    for _ in range(3):
        g.substep(0.0, 1.0, 1 / 24)
    s1 = g.save_state()
    np.testing.assert_array_equal(s1["x"], s0["x"])
    for k in ("F", "Jp", "mat", "emitter"):
        np.testing.assert_array_equal(s1[k], s0[k])


def test_reorder_does_not_change_the_physics():
    """Reordering every substep and never reordering give the same state after 50 substeps, up to the
    order in which float contributions are summed."""
    from mpm_plugin_gb300 import _abi

    d = domain(res=32)
    mats = [preset("jelly"), preset("sand_dry")]
    out = []
    for interval in (0, 1):
        g = gpu_solver(d, mats)
        add(g, box_particles((0.2, 0.3, 0.1), (0.45, 0.6, 0.4), d.dx, seed=1), 0, 0, (1.0, 0.0, 0.0))
        add(g, box_particles((0.5, 0.3, 0.0), (0.7, 0.6, 0.3), d.dx, seed=2), 1, 1)
        g.set_option(_abi.OPT_SORT_INTERVAL, interval)
        for _ in range(50):
            g.substep(2e-4, 1.0, 1 / 24)
        out.append(g.save_state())
    for k in ("x", "v", "F"):
        assert rel_err(out[1][k], out[0][k]) <= 1e-4, (k, rel_err(out[1][k], out[0][k]))


def test_errors_match_reference():
    d = domain(res=16)
    g = gpu_solver(d, [preset("jelly")])
    with pytest.raises(ValueError, match="material id out of range"):
        g.add_particles(np.zeros((2, 3)), np.zeros((2, 3)), np.array([0, 1]), np.zeros(2))
    with pytest.raises(ValueError, match="expected 0 collider transforms"):
        g.set_collider_transforms(np.eye(4)[None], np.eye(4)[None])
    g.add_particles(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0), np.zeros(0))  # empty is a no-op
    st = g.advance(1 / 24)
    assert (st.substeps, st.dt, st.removed) == (0, 1 / 24, 0)
    assert g.is_occupied(np.zeros((0, 3))).shape == (0,)


def test_conservation_accumulators_match_host_sums():
    """mpm_conservation (FP64 on the device) against float64 sums of the downloaded state, NaN skipped."""
    d = domain(res=32)
    mats = [preset("jelly"), preset("sand_dry")]
    g = gpu_solver(d, mats)
    add(g, box_particles((0.2, 0.3, 0.1), (0.4, 0.6, 0.4), d.dx, seed=1), 0, 0, (1.0, 0.0, 0.0))
    add(g, box_particles((0.5, 0.3, 0.0), (0.7, 0.6, 0.3), d.dx, seed=2), 1, 1, (0.0, -0.5, 0.2))
    for _ in range(10):
        g.substep(2e-4, 1.0, 1 / 24)
    st = g.save_state()
    st["x"][3] = np.nan
    g.load_state(st)
    c = g.conservation()
    pm = np.array([np.float32(m.density) * np.float32(d.dx ** 3 / 8) for m in mats], np.float64)[st["mat"]]
    ok = np.isfinite(st["x"]).all(1) & np.isfinite(st["v"]).all(1)
    m, x, v = pm[ok], st["x"][ok].astype(np.float64), st["v"][ok].astype(np.float64)
    assert c["non_finite"] == 1
    assert c["mass"] == pytest.approx(m.sum(), rel=1e-12)
    np.testing.assert_allclose(c["momentum"], (m[:, None] * v).sum(0), rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(c["com"], (m[:, None] * x).sum(0) / m.sum(), rtol=1e-10)
    assert c["ke"] == pytest.approx(0.5 * (m * (v * v).sum(1)).sum(), rel=1e-10)


def test_asynchronous_read_matches_synchronous_and_survives_the_next_advance():
    """read_begin / wait returns the state as save_state does at that moment, while the solver advances on;
    arrays of an earlier read stay intact after later reads."""
    d = domain(res=32)
    g = gpu_solver(d, [preset("jelly")])
    add(g, box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx, seed=1), 0, 0, (0.0, 0.5, 0.0))
    g.substep(2e-4, 1.0, 1 / 24)
    ref = g.save_state()
    pending = g.read_begin(tuple(ref))
    for _ in range(5):
        g.substep(2e-4, 1.0, 1 / 24)
    first = pending.wait()
    for k in ref:
        np.testing.assert_array_equal(first[k], ref[k])
    later = g.get_particles_async().wait()
    np.testing.assert_array_equal(later["x"], g.get_particles().positions)
    for k in ref:
        np.testing.assert_array_equal(first[k], ref[k])  # the earlier read's buffer was not reused


def test_run_substeps_equals_substeps_one_by_one():
    """mpm_run_substeps(dt, k) runs the same substeps as k calls of mpm_substep at s = (i + 1) / k."""
    d = domain(res=32)
    mats = [preset("jelly"), preset("sand_dry")]
    a, b = gpu_solver(d, mats), gpu_solver(d, mats)
    for s in (a, b):
        add(s, box_particles((0.3, 0.3, 0.1), (0.5, 0.6, 0.4), d.dx, seed=1), 0, 0, (1.0, 0.0, 0.0))
        add(s, box_particles((0.55, 0.3, 0.0), (0.7, 0.6, 0.3), d.dx, seed=2), 1, 1)
    a.run_substeps(2e-4, 12)
    for i in range(12):
        b.substep(2e-4, (i + 1) / 12, 12 * 2e-4)
    sa, sb = a.save_state(), b.save_state()
    for k in ("x", "v", "F"):
        assert rel_err(sa[k], sb[k]) <= 1e-5, (k, rel_err(sa[k], sb[k]))


def test_cooperative_substeps_match_kernel_by_kernel_substeps():
    """run_substeps in cooperative launches (forced, and with a collider) against the same substeps launched
    kernel by kernel, and an advance through the automatic choice for a small scene."""
    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    d, mats, groups, (cv, ct, xf) = mix_scene(res=64)
    out = []
    for coop in (0, 1):
        s = gpu_solver(d, mats)
        for pos, m, vel in groups:
            add(s, pos, m, m, vel)
        s.set_colliders([ColliderGeometry(MeshData(cv, ct), True, 0.5)])
        s.set_collider_transforms(xf[None], xf[None])
        s.set_option(_abi.OPT_COOP, coop)
        s.set_option(_abi.OPT_SORT_INTERVAL, 0)
        s.run_substeps(2e-4, 1)  # one substep the same way in both (and the colliders' voxel grids built)
        launches = s.launch_count()
        s.run_substeps(2e-4, 12)
        if coop:  # twelve substeps in one launch (and the collider poses of the twelve in one)
            assert s.launch_count() - launches <= 2
        out.append(s.save_state())
    for k in ("x", "v", "F"):
        assert rel_err(out[1][k], out[0][k]) <= 1e-5, (k, rel_err(out[1][k], out[0][k]))


def test_cooperative_barrier_gives_up_and_reports():
    """The grid barrier's bounded wait: with its arrival count preset so no CTA completes it, both CTAs give up
    after the spin limit and set the error flag; the context stays usable."""
    import ctypes as C

    d = domain(res=32)
    s = gpu_solver(d, [preset("jelly")])
    add(s, box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx))
    flag = C.c_int32(-1)
    assert s._lib.mpm_coop_barrier_selftest(s._h, 1, C.byref(flag)) == 0 and flag.value == 1
    assert s._lib.mpm_coop_barrier_selftest(s._h, 0, C.byref(flag)) == 0 and flag.value == 0
    st = s.advance(1 / 96)
    assert st.substeps > 0 and np.isfinite(s.save_state()["x"]).all()


def test_full_size_momentum_is_conserved_without_gravity_or_walls():
    """The 304k-particle mixed workload at full size, gravity off and collider off, for 200 substeps (the
    snowball in flight, no particle near a wall): P2G and G2P conserve momentum exactly in exact
    arithmetic (the affine terms sum to zero over a quadratic B-spline stencil), so the FP64 totals may move
    only by float rounding. A size-independent check at the metric's size, where the oracle is too slow."""
    from mpm_plugin_gb300.solver import Gb300Solver

    d, mats, groups, _ = mix_scene(res=128)
    g = Gb300Solver(d, mats, (0.0, 0.0, 0.0), 8, device="cuda:0")
    for pos, m, vel in groups:
        add(g, pos + np.float32([0.0, 0.0, 0.05]), m, m, vel)
    c0 = g.conservation()
    g.run_substeps(5e-5, 200)
    c1 = g.conservation()
    x = g.save_state()["x"]
    assert x.min() > d.dx * 3 and x.max() < 1 - d.dx * 3  # no wall contact
    assert c1["mass"] == c0["mass"]
    scale = c0["mass"] * 3.0  # total mass x the fastest initial speed
    assert np.linalg.norm(c1["momentum"] - c0["momentum"]) <= 1e-5 * scale, (c0["momentum"], c1["momentum"])


def test_pour_size_momentum_is_conserved():
    """The 256^3 pour's pile at its full size (7.45M particles, Drucker-Prager), lifted off the floor, gravity
    off, no collider, with a seeded swirl of velocities: 20 substeps conserve mass exactly and momentum up to
    float rounding (size-independent checks at the large workload's size)."""
    from mpm_plugin_gb300.interface import MaterialParams
    from mpm_plugin_gb300.solver import Gb300Solver
    from scenes import lattice_box

    d = domain(res=256)
    mats = [MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)]
    pile = lattice_box((0.2, 0.2, 0.2), (0.8, 0.8, 0.355), d.dx / 2, np.random.default_rng(3))
    rng = np.random.default_rng(4)
    c = pile.mean(0)
    vel = (np.cross(np.float32([0.0, 0.0, 1.0]), pile - c) + rng.normal(0, 0.1, pile.shape)).astype(np.float32)
    g = Gb300Solver(d, mats, (0.0, 0.0, 0.0), 8, device="cuda:0")
    z = np.zeros(len(pile), np.int32)
    g.add_particles(pile, vel, z, z)
    assert g.particle_count > 7_000_000
    c0 = g.conservation()
    g.run_substeps(1e-4, 20)
    c1 = g.conservation()
    assert c1["mass"] == c0["mass"]
    scale = c0["mass"] * float(np.abs(vel).max())
    assert np.linalg.norm(c1["momentum"] - c0["momentum"]) <= 1e-5 * scale, (c0["momentum"], c1["momentum"])
    g.close()


def test_whole_substep_timing():
    """MPM_OPT_KERNEL_TIMING 2 times whole substeps (events at the graph's two ends), 1 the kernel groups;
    neither changes the physics."""
    from mpm_plugin_gb300 import _abi

    d = domain(res=32)
    states = []
    for mode in (0, 1, 2):
        s = gpu_solver(d, [preset("jelly")])
        add(s, box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx, seed=3))
        s.set_option(_abi.OPT_KERNEL_TIMING, mode)
        for _ in range(5):
            s.substep(2e-4, 1.0, 1 / 24)
        groups = s.kernel_times()
        ms, count = s.substep_times(reset=True)  # (a reset clears both)
        if mode == 2:
            assert count == 5 and ms > 0 and all(c == 0 for _, c in groups.values())
        if mode == 1:
            assert count == 0 and groups["g2p"][1] == 5 and groups["p2g"][0] > 0
        states.append(s.save_state())
    for st in states[1:]:
        for k in ("x", "v", "F"):
            assert rel_err(st[k], states[0][k]) <= 1e-5

"""Two-grid mode (MPM_OPT_FUSED_P2G): G2P scatters each particle into the next substep's grid, so the next
substep's P2G reads no particle state. The physics must not change: every sequence of calls gives the same
state as in one-grid mode (float sums in another order: within 1e-5 relative, as two one-grid runs of the
same substeps), and the FP32 oracle agrees with it as with the one-grid mode.
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import add, box_particles, domain, mix_scene, perturbed_state, preset

from mpm_plugin_gb300 import _abi

pytestmark = pytest.mark.gpu


def _solver(d, mats):
    from mpm_plugin_gb300.solver import Gb300Solver

    return Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device="cuda:0")


def _mix(res=64, fused=True, sort_interval=4):
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

    d, mats, groups, (cv, ct, xf) = mix_scene(res=res)
    s = _solver(d, mats)
    for pos, m, vel in groups:
        add(s, pos, m, m, vel)
    s.set_colliders([ColliderGeometry(MeshData(cv, ct), True, 0.5)])
    s.set_collider_transforms(xf[None], xf[None])
    s.set_option(_abi.OPT_SORT_INTERVAL, sort_interval)
    s.set_option(_abi.OPT_FUSED_P2G, 1 if fused else 0)
    return s, d


def _close(a, b, keys=("x", "v", "C", "F", "Jp"), tol=1e-5, floor_c=None):
    for k in keys:
        e = rel_err(a[k], b[k], floor=floor_c) if (k == "C" and floor_c) else rel_err(a[k], b[k])
        assert e <= tol, (k, e)


def test_explicit_substeps_match_one_grid_mode():
    """Twelve explicit substeps with one dt (each scattering for the next), a collider and the periodic
    reorder in between, against the same substeps in one-grid mode."""
    out = []
    for fused in (False, True):
        s, d = _mix(fused=fused)
        for i in range(12):
            s.substep(2e-4, (i + 1) / 12, 12 * 2e-4)
        out.append(s.save_state())
    gnorm = float(np.linalg.norm(out[0]["v"]) / d.dx)
    _close(out[1], out[0], floor_c=gnorm)


def test_one_and_three_substeps_match_the_oracle():
    """The fused path against the FP32 oracle on the four-model scene: after one substep (P2G at the start, as
    always) and after three (the second and third take the grid the G2P before them scattered)."""
    from oracle.oracle import OracleSolver

    d = domain(res=32)
    mats = [preset("jelly"), preset("mashed_potato"), preset("sand_dry"), preset("snow_packed")]
    g = _solver(d, mats)
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=4)
    for i in range(4):
        pos = box_particles((0.1 + 0.2 * i, 0.3, 0.05), (0.25 + 0.2 * i, 0.6, 0.4), d.dx, seed=i)
        add(g, pos, i, i)
        add(o, pos, i, i)
    state = perturbed_state(g.save_state(), seed=11)
    g.load_state(state)
    o.load_state(state)
    g.set_option(_abi.OPT_FUSED_P2G, 1)
    g.set_option(_abi.OPT_SORT_INTERVAL, 0)
    o.frame_dt = 1 / 24
    for count in (1, 2):
        for _ in range(count):
            g.substep(2e-4, 1.0, 1 / 24)
            o.substep(2e-4, 1.0)
        out, ref = g.save_state(), o.save_state()
        gnorm = float(np.linalg.norm(ref["v"]) / d.dx)
        errs = {k: rel_err(out[k], ref[k], floor=gnorm) if k == "C" else rel_err(out[k], ref[k])
                for k in ("x", "v", "C", "F", "Jp")}
        print(count, {k: f"{e:.2e}" for k, e in errs.items()})
        for k, e in errs.items():
            assert e <= 1e-5, (count, k, e)


def test_run_substeps_and_advance_match_one_grid_mode():
    """Substeps of one advance (P2G only at the first, no scatter after the last): run_substeps against one-grid
    mode within 1e-5; a whole frame through advance with the same substep count and dt, and the invariants."""
    out, stats, inv = [], [], []
    for fused in (False, True):
        s, _ = _mix(fused=fused)
        s.run_substeps(2e-4, 12)
        out.append(s.save_state())
        st = s.advance(1 / 24)
        stats.append((st.substeps, st.dt, st.removed))
        c = s.conservation()
        inv.append(c)
    _close(out[1], out[0], keys=("x", "v", "F"))
    assert stats[0] == stats[1]
    a, b = inv
    for k in a:
        va, vb = np.asarray(a[k], np.float64), np.asarray(b[k], np.float64)
        assert np.linalg.norm(va - vb) <= 1e-4 * (np.linalg.norm(vb) + 1e-12), (k, a[k], b[k])


def test_a_scatter_for_a_substep_that_does_not_follow_is_dropped():
    """After an explicit substep (which scattered for a next one with its dt): another dt, an occupancy query
    (kept), new particles, a loaded state, an advance, a batch, deterministic mode and the option switched off and on, each against the
    same calls in one-grid mode."""
    from mpm_plugin_gb300.batch import Gb300Batch

    out = []
    for fused in (False, True):
        s, d = _mix(fused=fused, sort_interval=0)
        s.substep(2e-4, 1.0, 1 / 24)
        s.substep(1e-4, 1.0, 1 / 24)  # another dt
        s.substep(1e-4, 1.0, 1 / 24)
        # the emission path between explicit substeps: an occupancy query (no particle changes, the scatter
        # is kept) and then the free points added (the scatter is dropped)
        probe = box_particles((0.1, 0.1, 0.6), (0.2, 0.2, 0.7), d.dx, seed=5)
        assert not s.is_occupied(probe).any()
        s.substep(1e-4, 1.0, 1 / 24)
        add(s, probe, 0, 0)  # new particles
        s.substep(1e-4, 1.0, 1 / 24)
        state = s.save_state()
        s.substep(1e-4, 1.0, 1 / 24)
        s.load_state(state)  # back to the state before that substep
        s.substep(1e-4, 1.0, 1 / 24)
        s.run_substeps(1e-4, 3)
        s.substep(1e-4, 1.0, 1 / 24)
        s.set_option(_abi.OPT_DETERMINISTIC, 1)
        s.substep(1e-4, 1.0, 1 / 24)
        s.set_option(_abi.OPT_DETERMINISTIC, 0)
        s.substep(1e-4, 1.0, 1 / 24)
        s.set_option(_abi.OPT_FUSED_P2G, 0)
        s.substep(1e-4, 1.0, 1 / 24)
        s.set_option(_abi.OPT_FUSED_P2G, 1 if fused else 0)
        s.substep(1e-4, 1.0, 1 / 24)
        b = Gb300Batch([s])
        b.advance([1e-4 * 4])
        b.close()
        s.substep(1e-4, 1.0, 1 / 24)
        s.substep(1e-4, 1.0, 1 / 24)
        out.append(s.save_state())
    _close(out[1], out[0], keys=("x", "v", "F"))


def test_grid_read_back_and_memory():
    """read_grid gives the last substep's grid (not the one scattered for the next substep); the second grid
    is counted in the device memory and freed with the option."""
    grids, nbytes = [], []
    for fused in (False, True):
        s, _ = _mix(fused=fused)
        s.substep(2e-4, 1.0, 1 / 24)
        s.substep(2e-4, 1.0, 1 / 24)
        grids.append(s.read_grid())
        nbytes.append(s.device_bytes())
        if fused:
            s.set_option(_abi.OPT_FUSED_P2G, 0)
            assert s.device_bytes() == nbytes[0]
    m0, m1 = grids[0][..., 3], grids[1][..., 3]
    assert m0.sum() > 0
    np.testing.assert_allclose(m1, m0, rtol=0, atol=1e-5 * m0.max())
    cells = int(np.prod(grids[0].shape[:3]))
    assert nbytes[1] - nbytes[0] >= 16 * cells


def test_deterministic_mode_ignores_the_option():
    """Deterministic mode runs one grid whatever the option says: bit-identical to the option off."""
    out = []
    for fused in (False, True):
        s, _ = _mix(fused=fused, sort_interval=0)
        s.set_option(_abi.OPT_DETERMINISTIC, 1)
        for _ in range(4):
            s.substep(2e-4, 1.0, 1 / 24)
        out.append(s.save_state())
    for k in ("x", "v", "C", "F", "Jp"):
        np.testing.assert_array_equal(out[1][k], out[0][k])

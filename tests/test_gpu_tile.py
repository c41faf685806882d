"""Launch variants that must not change the physics (GPU): the TMA tile G2P (MPM_OPT_G2P_VARIANT 2) against
the plain G2P build and the oracle, P2G's block flags listed by a sweep (MPM_OPT_BLOCK_SWEEP) against P2G
listing the blocks itself, and several particles per thread (MPM_OPT_PARTICLES_PER_THREAD) against one.

Both builds run the same per-particle arithmetic in the same order; only where the inputs come from differs
(shared-memory tiles filled by cp.async.bulk.tensor, or global memory). In deterministic mode (P2G sums in
fixed point, independent of atomic order) the two must give bit-identical states: with the particles in
grid-block order (reorder every substep or every few), where nearly every particle's stencil comes from a
staged grid box, and in the sampler's order (no reorder), where many chunks span more base blocks than the
kernel stages and those particles gather from global memory.
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import add, box_particles, domain, mix_scene, perturbed_state, preset

from mpm_plugin_gb300 import _abi

pytestmark = pytest.mark.gpu


def _mix(variant, sort_interval, res=128, deterministic=True, block_sweep=0, ppt=1):
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver

    d, mats, groups, (cv, ct, xf) = mix_scene(res=res)
    s = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device="cuda:0")
    for pos, m, vel in groups:
        add(s, pos, m, m, vel)
    s.set_colliders([ColliderGeometry(MeshData(cv, ct), True, 0.5)])
    s.set_collider_transforms(xf[None], xf[None])
    s.set_option(_abi.OPT_DETERMINISTIC, int(deterministic))
    s.set_option(_abi.OPT_SORT_INTERVAL, sort_interval)
    s.set_option(_abi.OPT_G2P_VARIANT, variant)
    s.set_option(_abi.OPT_BLOCK_SWEEP, block_sweep)
    s.set_option(_abi.OPT_PARTICLES_PER_THREAD, ppt)
    return s, d


@pytest.mark.parametrize("variant,sort_interval", [(2, 1), (2, 4), (2, 0), (1, 4), (3, 0)])
def test_tile_g2p_is_bit_identical_to_the_plain_build(variant, sort_interval):
    """The tile build (2), and the uncapped (1) and 80-register (3) plain builds, against the default
    64-register plain build."""
    out = []
    for variant in (0, variant):
        s, _ = _mix(variant, sort_interval)
        s.run_substeps(5e-5, 12)
        for _ in range(3):
            s.substep(5e-5, 1.0, 1 / 24)
        st = s.advance(1 / 24)
        out.append((s.save_state(), (st.substeps, st.dt, st.removed)))
        s.close()
    (a, sa), (b, sb) = out
    assert sa == sb
    for k in ("x", "v", "C", "F", "Jp", "mat", "emitter"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_tile_g2p_matches_the_oracle():
    """One substep of the four-model scene from a perturbed state (particles in the sampler's order)."""
    from mpm_plugin_gb300.solver import Gb300Solver
    from oracle.oracle import OracleSolver

    d = domain(res=32)
    mats = [preset("jelly"), preset("mashed_potato"), preset("sand_dry"), preset("snow_packed")]
    g = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device="cuda:0")
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=4)
    for i in range(4):
        pos = box_particles((0.1 + 0.2 * i, 0.3, 0.05), (0.25 + 0.2 * i, 0.6, 0.4), d.dx, seed=i)
        add(g, pos, i, i)
        add(o, pos, i, i)
    state = perturbed_state(g.save_state(), seed=11)
    g.load_state(state)
    o.load_state(state)
    g.set_option(_abi.OPT_G2P_VARIANT, 2)
    g.substep(2e-4, 1.0, 1 / 24)
    o.frame_dt = 1 / 24
    o.substep(2e-4, 1.0)
    out, ref = g.save_state(), o.save_state()
    gnorm = float(np.linalg.norm(ref["v"]) / d.dx)
    for k in ("x", "v", "C", "F", "Jp"):
        e = rel_err(out[k], ref[k], floor=gnorm if k == "C" else 0.0)
        assert e <= 1e-5, (k, e)


def test_tile_g2p_at_the_pour_size_conserves_momentum():
    """The 256^3 pour's pile (7.45M particles, 29k chunks over the persistent CTAs) in grid-block order: 20
    substeps without gravity or walls conserve mass exactly and momentum to float rounding, as the plain
    build does."""
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
    g.set_option(_abi.OPT_G2P_VARIANT, 2)
    g.set_option(_abi.OPT_SORT_INTERVAL, 4)
    c0 = g.conservation()
    g.run_substeps(1e-4, 20)
    c1 = g.conservation()
    assert c1["mass"] == c0["mass"] and c1["non_finite"] == 0
    scale = c0["mass"] * float(np.abs(vel).max())
    assert np.linalg.norm(c1["momentum"] - c0["momentum"]) <= 1e-5 * scale, (c0["momentum"], c1["momentum"])
    g.close()


@pytest.mark.parametrize("variant,sort_interval", [(0, 0), (2, 4)])
def test_block_sweep_is_bit_identical_to_listing_in_p2g(variant, sort_interval):
    """Deterministic mode: P2G flagging blocks for k_list_blocks gives the state P2G listing them does, over
    graph-replayed substeps, explicit substeps and an advance with the CFL step, a collider in the scene."""
    out = []
    for sweep in (0, 1):
        s, _ = _mix(variant, sort_interval, block_sweep=sweep)
        s.run_substeps(5e-5, 12)
        for _ in range(3):
            s.substep(5e-5, 1.0, 1 / 24)
        st = s.advance(1 / 24)
        out.append((s.save_state(), (st.substeps, st.dt, st.removed), s.read_grid()))
        s.close()
    (a, sa, ga), (b, sb, gb) = out
    assert sa == sb
    np.testing.assert_array_equal(ga, gb)
    for k in ("x", "v", "C", "F", "Jp"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("ppt,fused", [(2, 0), (4, 0), (8, 0), (4, 1)])
def test_particles_per_thread_do_not_change_the_state(ppt, fused):
    """Deterministic mode: P2G and G2P with CTAs that take several chunks each give the state of one CTA per
    chunk, bit for bit, over graph-replayed substeps, explicit substeps and an advance; in the default mode
    (float atomics, any order) and in two-grid mode, within 1e-5 after one substep."""
    out = []
    for k in (1, ppt):
        s, _ = _mix(0, 4, ppt=k)
        s.run_substeps(5e-5, 12)
        for _ in range(3):
            s.substep(5e-5, 1.0, 1 / 24)
        st = s.advance(1 / 24)
        out.append((s.save_state(), (st.substeps, st.dt, st.removed)))
        s.close()
    (a, sa), (b, sb) = out
    assert sa == sb
    for k in ("x", "v", "C", "F", "Jp"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    out = []
    for k in (1, ppt):
        s, d = _mix(0, 0, deterministic=False, ppt=k)
        s.set_option(_abi.OPT_FUSED_P2G, fused)
        s.run_substeps(5e-5, 3)
        out.append(s.save_state())
        s.close()
    # C against the velocity-gradient scale (|v| / dx): near rest it is the rounding of sums in any order
    gnorm = float(np.linalg.norm(out[0]["v"])) / d.dx
    for k in ("x", "v", "C", "F", "Jp"):
        assert rel_err(out[1][k], out[0][k], floor=gnorm if k == "C" else 0.0) <= 1e-5, k


@pytest.mark.parametrize("sort_interval", [0, 4])
def test_p2g_merge_along_z_matches_one_reduction_per_leader(sort_interval):
    """P2G with the leaders' sums merged along z (MPM_OPT_P2G_MERGE 1) against one reduction per node and
    leader (0): the grid after a substep (each node's mass, and the total against the particles' mass: no
    contribution lost or added twice) and the particle state after three agree within float summation order
    (1e-5), in the sampler's order and after reorders."""
    out = []
    for merge in (0, 1):
        s, d = _mix(0, sort_interval, deterministic=False)
        s.set_option(_abi.OPT_P2G_MERGE, merge)
        mass = s.conservation()["mass"]
        s.substep(5e-5, 1.0, 1 / 24)
        grid = s.read_grid()
        assert abs(grid[..., 3].astype(np.float64).sum() - mass) <= 1e-5 * mass
        s.run_substeps(5e-5, 2)
        out.append((grid, s.save_state()))
        s.close()
    (g0, a), (g1, b) = out
    assert rel_err(g1[..., 3], g0[..., 3]) <= 1e-5
    assert rel_err(g1, g0) <= 1e-5
    gnorm = float(np.linalg.norm(a["v"])) / d.dx
    for k in ("x", "v", "C", "F", "Jp"):
        assert rel_err(b[k], a[k], floor=gnorm if k == "C" else 0.0) <= 1e-5, k

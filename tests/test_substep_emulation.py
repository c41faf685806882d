"""The CUDA backend's substep code (mpm_substep.cuh), compiled for the host, against the reference fixtures.

Same per-particle and per-node functions the kernels run, executed one item after another on the CPU (no
fused multiply-adds, sequential accumulation), so this checks the kernel logic without a GPU.
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import SOLVER_CASES, Case, rel_err
from device_math import SubstepEmulator

SUBSTEP_CASES = [n for n in SOLVER_CASES if Case(n).action["kind"] == "substep"]


@pytest.mark.parametrize("name", SUBSTEP_CASES)
def test_emulated_substep_matches_reference(name):
    case = Case(name)
    a = case.action
    e = SubstepEmulator(case.domain, case.materials, case.gravity, case.ppc)
    e.load_state(case.state("in"))
    e.set_colliders(case.colliders())
    if case.transforms() is not None:
        e.set_collider_transforms(*case.transforms())
    for k in range(a.get("count", 1)):
        e.substep(a["dt"], a["s"][k] if isinstance(a["s"], list) else a["s"], a["frame_dt"])
    out, ref = e.save_state(), case.state("out")
    for k in ("x", "v", "C", "F", "Jp"):
        assert rel_err(out[k], ref[k]) <= 1e-5, (k, rel_err(out[k], ref[k]))


def test_stored_stress_matches_stress_of_stored_f():
    """The stress G2P stores (from the trial F's SVD after the return mapping) equals the stress of the
    stored F decomposed again, which is what the reference's next P2G computes."""
    case = Case("models_substep")
    a = case.action
    e = SubstepEmulator(case.domain, case.materials, case.gravity, case.ppc)
    e.load_state(case.state("in"))
    for _ in range(3):
        e.substep(a["dt"], a["s"], a["frame_dt"])
    kept, fresh = e.state["tau"], e.stress_of_state()
    scale = np.abs(fresh).max()
    assert scale > 0
    assert np.abs(kept - fresh).max() <= 1e-5 * scale, np.abs(kept - fresh).max() / scale


def test_emulated_grid_matches_oracle_grid():
    """Node by node: mass and velocity after the grid update and collider contact."""
    from oracle.oracle import OracleSolver

    case = Case("collider_sphere_substep")
    a = case.action
    e = SubstepEmulator(case.domain, case.materials, case.gravity, case.ppc)
    o = OracleSolver(case.domain, case.materials, case.gravity, case.ppc)
    for s in (e, o):
        s.load_state(case.state("in"))
        s.set_colliders(case.colliders())
        s.set_collider_transforms(*case.transforms())
    e.substep(a["dt"], a["s"], a["frame_dt"])
    o.frame_dt = a["frame_dt"]
    o.substep(a["dt"], a["s"])
    ge, go = e.read_grid(), o.grid
    np.testing.assert_allclose(ge[..., 3], go[..., 3], rtol=0, atol=1e-6 * go[..., 3].max())
    m = go[..., 3] > 0
    dv = np.linalg.norm(ge[..., :3] - go[..., :3], axis=-1)[m]
    assert dv.max() <= 1e-5 * np.abs(go[..., :3][m]).max()

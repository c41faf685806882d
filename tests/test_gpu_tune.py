"""The autotuner on the GPU: it measures every candidate launch choice on the solver's own scene, leaves the
scene's state where it was, caches the choice per GPU and workload class, and a tuned solver computes the
same physics."""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import add, box_particles, domain, preset

pytestmark = pytest.mark.gpu


def _solver():
    from mpm_plugin_gb300 import create

    d = domain(res=48)
    s = create(domain=d, materials=[preset("sand_dry")], gravity=(0.0, 0.0, -9.81), device="cuda:0")
    add(s, box_particles((0.3, 0.3, 0.0), (0.7, 0.7, 0.25), d.dx, seed=5), 0, 0, (0.3, 0.0, 0.0))
    return s


def test_tune_solver_restores_state_and_caches(tmp_path):
    from mpm_plugin_gb300 import tune

    path = tmp_path / "autotune.json"
    s = _solver()
    before = s.save_state()
    cfg = tune.tune_solver(s, 2e-4, substeps=8, path=path)
    assert not cfg["cached"] and cfg["trials"] >= 6 and cfg["seconds_per_substep"] > 0
    after = s.save_state()
    for k in ("x", "v", "C", "F", "Jp", "mat", "emitter"):
        np.testing.assert_array_equal(after[k], before[k])
    again = tune.tune_solver(_solver(), 2e-4, substeps=8, path=path)
    assert again["cached"] and {k: again[k] for k in tune.DEFAULTS} == {k: cfg[k] for k in tune.DEFAULTS}
    ref = _solver()
    for _ in range(20):
        s.substep(2e-4, 1.0, 1 / 24)
        ref.substep(2e-4, 1.0, 1 / 24)
    assert rel_err(s.save_state()["x"], ref.save_state()["x"]) <= 1e-4


def test_tune_solver_on_run_substeps_restores_state_and_caches_apart(tmp_path):
    """runs=True times run_substeps calls: the state is restored, the choice is cached under its own key."""
    from mpm_plugin_gb300 import tune

    path = tmp_path / "autotune.json"
    s = _solver()
    before = s.save_state()
    cfg = tune.tune_solver(s, 2e-4, substeps=16, path=path, runs=True)
    assert not cfg["cached"] and cfg["seconds_per_substep"] > 0 and "fused_p2g" in cfg
    after = s.save_state()
    for k in ("x", "v", "C", "F", "Jp", "mat", "emitter"):
        np.testing.assert_array_equal(after[k], before[k])
    assert tune.tune_solver(_solver(), 2e-4, substeps=16, path=path, runs=True)["cached"]
    assert not tune.tune_solver(_solver(), 2e-4, substeps=8, path=path)["cached"]  # the other key


@pytest.mark.parametrize("variant,ctas_per_sm,group,pdl,tile", [(0, 4, 1, 0, 0), (1, 16, 4, 1, 0), (1, 8, 32, 0, 1),
                                                              (0, 16, 8, 1, 1), (0, 8, 32, 1, 0), (1, 4, 8, 0, 1)])
def test_every_launch_choice_gives_the_same_physics(variant, ctas_per_sm, group, pdl, tile):
    from mpm_plugin_gb300 import _abi

    s, ref = _solver(), _solver()
    ref.set_option(_abi.OPT_PDL, 0)
    s.set_option(_abi.OPT_PDL, pdl)
    s.set_option(_abi.OPT_P2G_TILE, tile)
    s.set_option(_abi.OPT_G2P_VARIANT, variant)
    s.set_option(_abi.OPT_LIST_CTAS, ctas_per_sm * 152)
    s.set_option(_abi.OPT_P2G_GROUP, group)
    for _ in range(10):
        s.substep(2e-4, 1.0, 1 / 24)
        ref.substep(2e-4, 1.0, 1 / 24)
    a, b = s.save_state(), ref.save_state()
    for k in ("x", "v", "F"):
        assert rel_err(a[k], b[k]) <= 1e-5, (k, rel_err(a[k], b[k]))

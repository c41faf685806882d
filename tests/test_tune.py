"""Autotuner host logic on the CPU: the coordinate-descent search, workload classes and the cache file."""

from __future__ import annotations

from mpm_plugin_gb300 import tune


def test_search_finds_the_separable_optimum_and_keeps_defaults_on_ties():
    best_cfg = {"sort_interval": 8, "g2p_variant": 1, "list_ctas_per_sm": 4, "p2g_group": 8, "pdl": 1,
                "p2g_merge": 0}
    cost = {"sort_interval": {0: 3.0, 2: 1.5, 4: 1.0, 8: 0.5, 16: 0.9},
            "g2p_variant": {0: 1.0, 1: 0.6}, "list_ctas_per_sm": {2: 0.25, 4: 0.2, 8: 0.3, 16: 0.5},
            "p2g_group": {1: 0.9, 4: 0.5, 8: 0.4, 32: 0.6}, "pdl": {0: 0.3, 1: 0.1}, "p2g_merge": {0: 0.1, 1: 0.3}}
    calls = []

    def measure(cfg):
        calls.append(cfg)
        return sum(cost[k][v] for k, v in cfg.items())

    best, t, trials = tune.search(measure)
    assert best == best_cfg
    assert t == sum(cost[k][v] for k, v in best_cfg.items())
    assert len(trials) == len(calls) == 1 + sum(len(v) - 1 for v in tune.CANDIDATES.values())
    flat, _, _ = tune.search(lambda cfg: 1.0)  # nothing is 2 % better: the defaults stay
    assert flat == tune.DEFAULTS


def test_workload_classes_round_to_powers_of_two():
    assert tune.workload_key(128, 304_322, True) == "res128|n262144|col1|det0"
    assert tune.workload_key(100, 300_000, False, True) == tune.workload_key(128, 270_000, False, True)
    assert tune.workload_key(64, 1000, False) != tune.workload_key(128, 1000, False)


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "autotune.json"
    assert tune.load_cache(path) == {}
    tune.store_cache({"gpu|152": {"res128|n262144|col1|det0": tune.DEFAULTS}}, path)
    assert tune.load_cache(path)["gpu|152"]["res128|n262144|col1|det0"] == tune.DEFAULTS
    monkeypatch.setenv("MPM_GB300_TUNE_CACHE", str(path))
    assert tune.cache_path() == path
    path.write_text("{not json")
    assert tune.load_cache(path) == {}


class _FakeSolver:
    """The parts of Gb300Solver the tuner uses; a run_substeps call advances a counter standing in for the
    scene's state, and its cost depends on the options set and on how far the scene has moved on."""

    device = "cuda:0"
    particle_count = 32_768
    _n_colliders = 0

    def grid_dims(self):
        return (70, 70, 70)

    def __init__(self):
        self.state, self.opts, self.loads = 0, {}, 0

    def save_state(self):
        return {"step": self.state}

    def load_state(self, st):
        self.state = st["step"]
        self.loads += 1

    def set_option(self, option, value):
        self.opts[option] = value

    def run_substeps(self, dt, count):
        self.state += count


def test_run_substeps_tuning_restores_the_state_per_trial_and_keeps_its_own_key(tmp_path, monkeypatch):
    import time

    import torch

    from mpm_plugin_gb300 import _abi

    clock = {"t": 0.0}
    monkeypatch.setattr(tune, "gpu_key", lambda device: ("gpu|152", 152))
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(time, "perf_counter", lambda: clock["t"])
    s = _FakeSolver()
    real_run = s.run_substeps

    def run(dt, count):  # 1 s per substep, 3 s with the two-grid mode, plus the scene's age if not restored
        clock["t"] += count * (3.0 if s.opts.get(_abi.OPT_FUSED_P2G) else 1.0) + s.state
        real_run(dt, count)

    s.run_substeps = run
    path = tmp_path / "autotune.json"
    cfg = tune.tune_solver(s, 1e-4, 1e-4, substeps=10, path=path, runs=True)
    trials = cfg["trials"]
    assert s.loads == trials + 1  # before every trial, and once at the end
    assert s.state == 0
    assert cfg["fused_p2g"] == 0 and s.opts[_abi.OPT_FUSED_P2G] == 0
    assert list(tune.load_cache(path)["gpu|152"]) == [tune.workload_key(64, 32_768, False) + "|runs"]
    assert tune.tune_solver(_FakeSolver(), 1e-4, 1e-4, path=path, runs=True)["cached"]


def test_the_two_grid_knob_is_searched_last_for_a_solver():
    """fused_p2g is the last knob of the descent (it must beat the tuned one-grid choice); the solver-only
    knobs come after the batch knobs; the joint tile-G2P-with-reorder trials keep one grid."""
    assert tune.SOLVER_ORDER[-1] == "fused_p2g" and tune.SOLVER_ORDER[:len(tune.KNOB_ORDER)] == tune.KNOB_ORDER
    assert tune.SOLVER_DEFAULTS["fused_p2g"] == 0 and "fused_p2g" not in tune.DEFAULTS
    assert tune.SOLVER_DEFAULTS["block_sweep"] == 0 and "block_sweep" not in tune.DEFAULTS
    assert all(o["g2p_variant"] == 2 and o["sort_interval"] > 0 and o["fused_p2g"] == 0 for o in tune.SOLVER_JOINT)


def test_joint_overrides_are_tried_from_the_best_of_the_descent():
    times = {(0, 0): 1.0, (1, 0): 0.9, (2, 0): 1.2, (0, 4): 1.1, (1, 4): 0.95, (2, 4): 0.5}

    def measure(cfg):
        return times.get((cfg["a"], cfg["b"]), 2.0)

    best, t, trials = tune.search(measure, {"a": (0, 1, 2), "b": (0, 4)}, {"a": 0, "b": 0}, ("a", "b"),
                                  joint=({"a": 2, "b": 4},))
    assert best == {"a": 2, "b": 4} and t == 0.5  # one knob at a time stops at (1, 0)
    assert len(trials) == 5


def test_joint_overrides_need_the_larger_gain():
    """A joint override within JOINT_MIN_GAIN of the descent's best is not taken (its window is noisier than
    the gain)."""
    times = {(0, 0): 1.0, (1, 0): 0.9, (2, 4): 0.9 * (1.0 - tune.JOINT_MIN_GAIN / 2)}
    best, t, _ = tune.search(lambda cfg: times.get((cfg["a"], cfg["b"]), 2.0), {"a": (0, 1), "b": (0,)},
                             {"a": 0, "b": 0}, ("a", "b"), joint=({"a": 2, "b": 4},))
    assert best == {"a": 1, "b": 0} and t == 0.9

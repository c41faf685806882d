"""Autotuner host logic on the CPU: the coordinate-descent search, workload classes and the cache file."""

from __future__ import annotations

from mpm_plugin_gb300 import tune


def test_search_finds_the_separable_optimum_and_keeps_defaults_on_ties():
    best_cfg = {"sort_interval": 8, "g2p_variant": 1, "list_ctas_per_sm": 4, "p2g_group": 8, "pdl": 1}
    cost = {"sort_interval": {0: 3.0, 2: 1.5, 4: 1.0, 8: 0.5, 16: 0.9},
            "g2p_variant": {0: 1.0, 1: 0.6}, "list_ctas_per_sm": {2: 0.25, 4: 0.2, 8: 0.3, 16: 0.5},
            "p2g_group": {1: 0.9, 4: 0.5, 8: 0.4, 32: 0.6}, "pdl": {0: 0.3, 1: 0.1}}
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

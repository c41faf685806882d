"""Autotuner: picks a solver's (or batch's) launch choices by timing them on the workload itself, and caches
the choice per GPU and workload class.

Knobs (C options of include/mpm_gb300.h):
  sort_interval      reorder of the particles by grid node after every N substeps (0: never);
  g2p_variant        G2P build: 0 capped at 80 registers (3 CTAs of 256 per SM), 1 uncapped, 2 (a solver) the
                     persistent tile G2P, its inputs and grid boxes brought into shared memory by TMA;
  list_ctas_per_sm   CTAs per SM of the kernels that walk the active-block and candidate lists;
  p2g_group          P2G sums same-cell lanes within aligned groups of this many lanes (1 .. 32);
  pdl                programmatic dependent launch of the substep kernels (1) or plain stream order (0);
  block_sweep        (a solver) P2G flags the blocks it touches and a sweep lists them (1), or P2G lists them
                     with atomics (0);
  fused_p2g          (a solver, outside deterministic mode) two grids, G2P scattering each particle into the
                     next substep's grid (1), or P2G on its own at the start of every substep (0).

The shared-memory tile P2G (MPM_OPT_P2G_TILE) is not searched: it was slower than the warp segments on the
unsorted mixed workload and on the 256^3 pour, and in a short tuning window it could look faster.

Search: coordinate descent from the defaults, one knob at a time over its candidates with the others fixed,
keeping a change only when it is at least 2 % faster. A configuration is timed by CUDA events the solver
records at the two ends of each substep (MPM_OPT_KERNEL_TIMING 2, so the kernels inside stay chained as
untimed) over `substeps` substeps after 3 warm-up substeps; or, for a workload that runs as run_substeps
calls (runs=True), by the host clock around one run_substeps call of `substeps` substeps (eight substeps
per graph launch, chained across substeps), each trial from the saved state. A small scene's choice differs between the two: with one
substep per graph the graph launch hides what 1,216 near-idle work-list CTAs cost, with eight it does not. The solver's state is saved before and loaded back after, so tuning does not advance the bake
(a load recomputes the stored stress from F, a last-bit change).

Cache: JSON at $MPM_GB300_TUNE_CACHE or ~/.cache/mpm_plugin_gb300/autotune.json, keyed by the GPU (name,
SM count) and the workload class (grid resolution and particle count rounded to powers of two, colliders,
deterministic mode).
"""

from __future__ import annotations

import json
import math
import os
from pathlib import Path

from mpm_plugin_gb300 import _abi

DEFAULTS = {"sort_interval": 0, "g2p_variant": 0, "list_ctas_per_sm": 8, "p2g_group": 32, "pdl": 1, "p2g_merge": 1}
CANDIDATES = {"sort_interval": (0, 2, 4, 8, 16), "g2p_variant": (0, 1), "list_ctas_per_sm": (2, 4, 8, 16),
              "p2g_group": (1, 4, 8, 32), "pdl": (0, 1), "p2g_merge": (1, 0)}
KNOB_ORDER = ("g2p_variant", "sort_interval", "p2g_group", "list_ctas_per_sm", "pdl", "p2g_merge")
MIN_GAIN = 0.02
# A joint override (the tile G2P with a sort interval) has to win by more: on the 256^3 pour a 12-substep
# window preferred the tile build by 2-3 % and the frame then ran 12 % slower (measured).
JOINT_MIN_GAIN = 0.05
# A single solver also chooses between the one- and two-grid substeps, last: the two-grid mode has to beat
# the tuned one-grid choice. (Searched first, on the 256^3 pour it beat the untuned defaults, the descent
# then never reached the reorder that makes one grid faster, and a frame took 1.3x as long: measured.)
SOLVER_DEFAULTS = {**DEFAULTS, "block_sweep": 0, "ppt": 1, "fused_p2g": 0}
SOLVER_CANDIDATES = {**CANDIDATES, "g2p_variant": (0, 1, 2, 3), "block_sweep": (0, 1), "ppt": (1, 2, 4),
                     "fused_p2g": (0, 1)}
SOLVER_ORDER = KNOB_ORDER + ("block_sweep", "ppt", "fused_p2g")
# The tile G2P (g2p_variant 2) stages a chunk's grid boxes in shared memory, which pays when the particles are
# in grid-block order, i.e. with a periodic reorder: the two knobs are also tried together, from the best
# configuration of the descent (one knob at a time would try the tile G2P only at the sort interval then set).
SOLVER_JOINT = tuple({"g2p_variant": 2, "sort_interval": k, "fused_p2g": 0} for k in (1, 2, 4, 8, 16))


def cache_path() -> Path:
    env = os.environ.get("MPM_GB300_TUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "mpm_plugin_gb300" / "autotune.json"


def gpu_key(device: str = "cuda:0") -> tuple[str, int]:
    import torch

    p = torch.cuda.get_device_properties(torch.device(device))
    return f"{p.name}|{p.multi_processor_count}", int(p.multi_processor_count)


def workload_key(resolution: int, particles: int, colliders: bool, deterministic: bool = False) -> str:
    r = 2 ** round(math.log2(max(resolution, 1)))
    n = 2 ** round(math.log2(max(particles, 1)))
    return f"res{r}|n{n}|col{int(bool(colliders))}|det{int(bool(deterministic))}"


def load_cache(path: Path | None = None) -> dict:
    path = path or cache_path()
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def store_cache(cache: dict, path: Path | None = None) -> None:
    path = Path(path or cache_path())
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    tmp.replace(path)


def apply(target, cfg: dict, sms: int, solver: bool = False) -> None:
    """Set a configuration on a Gb300Solver (solver=True) or Gb300Batch. A solver always gets a grid mode: a
    configuration without the fused_p2g knob (one cached before the knob existed, or a deterministic one)
    means one grid, the mode it was measured in."""
    target.set_option(_abi.OPT_SORT_INTERVAL, int(cfg["sort_interval"]))
    target.set_option(_abi.OPT_G2P_VARIANT, int(cfg["g2p_variant"]))
    target.set_option(_abi.OPT_LIST_CTAS, int(cfg["list_ctas_per_sm"]) * sms)
    target.set_option(_abi.OPT_P2G_GROUP, int(cfg.get("p2g_group", 32)))
    target.set_option(_abi.OPT_PDL, int(cfg.get("pdl", 1)))
    target.set_option(_abi.OPT_P2G_TILE, int(cfg.get("p2g_tile", 0)))
    target.set_option(_abi.OPT_P2G_MERGE, int(cfg.get("p2g_merge", 1)))
    if solver:
        target.set_option(_abi.OPT_BLOCK_SWEEP, int(cfg.get("block_sweep", 0)))
        target.set_option(_abi.OPT_PARTICLES_PER_THREAD, int(cfg.get("ppt", 1)))
        target.set_option(_abi.OPT_FUSED_P2G, int(cfg.get("fused_p2g", 0)))


def search(measure, candidates=CANDIDATES, defaults=DEFAULTS, order=KNOB_ORDER, min_gain=MIN_GAIN, joint=(),
           joint_min_gain=JOINT_MIN_GAIN):
    """Coordinate descent: measure(cfg) -> seconds (lower is better), then each of the `joint` overrides (several
    knobs at once) applied to the best so far, kept only when it gains joint_min_gain. Returns (best cfg, its
    time, trials)."""
    best = dict(defaults)
    best_t = measure(best)
    trials = [(dict(best), best_t)]
    seen = {tuple(sorted(best.items()))}
    for knob in order:
        for value in candidates[knob]:
            cfg = {**best, knob: value}
            key = tuple(sorted(cfg.items()))
            if key in seen:
                continue
            seen.add(key)
            t = measure(cfg)
            trials.append((cfg, t))
            if t < best_t * (1.0 - min_gain):
                best, best_t = cfg, t
    base = dict(best)
    for over in joint:
        cfg = {**base, **over}
        key = tuple(sorted(cfg.items()))
        if key in seen:
            continue
        seen.add(key)
        t = measure(cfg)
        trials.append((cfg, t))
        if t < best_t * (1.0 - joint_min_gain):
            best, best_t = cfg, t
    return best, best_t, trials


def _time_solver(solver, cfg, sms, dt, frame_dt, substeps):
    apply(solver, cfg, sms, solver=True)
    for _ in range(3):
        solver.substep(dt, 1.0, frame_dt)
    solver.set_option(_abi.OPT_KERNEL_TIMING, 2)  # events at the two ends of each substep
    solver.substep_times(reset=True)
    for _ in range(substeps):
        solver.substep(dt, 1.0, frame_dt)
    ms, _ = solver.substep_times(reset=True)
    solver.set_option(_abi.OPT_KERNEL_TIMING, 0)
    return ms / 1e3 / substeps


def _time_runs(solver, cfg, sms, dt, substeps, repeats=3):
    import time

    import torch

    apply(solver, cfg, sms, solver=True)
    solver.run_substeps(dt, substeps)  # graphs captured
    best = float("inf")
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.run_substeps(dt, substeps)  # returns once its substeps are done
        best = min(best, time.perf_counter() - t0)
    return best / substeps


def tune_solver(solver, dt: float, frame_dt: float = 1 / 24, substeps: int = 20, path: Path | None = None,
                force: bool = False, deterministic: bool = False, runs: bool = False) -> dict:
    """Choose and set the solver's launch choices for its current scene; returns the configuration with
    ``cached`` (whether it came from the cache) and, when measured, ``seconds_per_substep``. runs: time
    run_substeps calls (the way a fixed-dt workload of many substeps per call runs) instead of single
    substeps."""
    gkey, sms = gpu_key(solver.device)
    wkey = workload_key(max(solver.grid_dims()) - 6, solver.particle_count, solver._n_colliders > 0, deterministic)
    if runs:
        wkey += "|runs"
    cache = load_cache(path)
    hit = cache.get(gkey, {}).get(wkey)
    if hit and not force:
        apply(solver, hit, sms, solver=True)
        return {**hit, "cached": True}
    snapshot = solver.save_state()
    if runs:  # every trial from the same state: thousands of substeps per trial move the scene on
        def measure(cfg):
            solver.load_state(snapshot)
            return _time_runs(solver, cfg, sms, dt, substeps)
    else:
        measure = lambda cfg: _time_solver(solver, cfg, sms, dt, frame_dt, substeps)  # noqa: E731
    if deterministic:  # one grid whatever fused_p2g says: that knob is not searched (nor set) there
        best, best_t, trials = search(measure, {k: v for k, v in SOLVER_CANDIDATES.items() if k != "fused_p2g"},
                                      {k: v for k, v in SOLVER_DEFAULTS.items() if k != "fused_p2g"},
                                      tuple(k for k in SOLVER_ORDER if k != "fused_p2g"),
                                      joint=tuple({k: v for k, v in o.items() if k != "fused_p2g"} for o in SOLVER_JOINT))
    else:
        best, best_t, trials = search(measure, SOLVER_CANDIDATES, SOLVER_DEFAULTS, SOLVER_ORDER, joint=SOLVER_JOINT)
    solver.load_state(snapshot)
    apply(solver, best, sms, solver=True)
    cache.setdefault(gkey, {})[wkey] = best
    store_cache(cache, path)
    return {**best, "cached": False, "seconds_per_substep": best_t, "trials": len(trials)}


def tune_batch(batch, frame_dt: float, frames: int = 2, path: Path | None = None, force: bool = False) -> dict:
    """The same for a batch, timing whole batched frames; every scene's state is restored afterwards."""
    import time

    import torch

    scenes = batch.scenes
    gkey, sms = gpu_key(scenes[0].device)
    n = sum(s.particle_count for s in scenes)
    res = max(max(s.grid_dims()) - 6 for s in scenes)
    wkey = "batch|" + workload_key(res, n, any(s._n_colliders > 0 for s in scenes)) + f"|scenes{len(scenes)}"
    cache = load_cache(path)
    hit = cache.get(gkey, {}).get(wkey)
    if hit and not force:
        apply(batch, hit, sms)
        return {**hit, "cached": True}
    snapshots = [s.save_state() for s in scenes]

    def measure(cfg):
        apply(batch, cfg, sms)
        batch.advance(frame_dt)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(frames):
            batch.advance(frame_dt)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / frames

    best, best_t, trials = search(measure)
    for s, st in zip(scenes, snapshots):
        s.load_state(st)
    apply(batch, best, sms)
    cache.setdefault(gkey, {})[wkey] = best
    store_cache(cache, path)
    return {**best, "cached": False, "seconds_per_frame": best_t, "trials": len(trials)}

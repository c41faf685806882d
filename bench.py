"""Throughput of the gb300 MLS-MPM substep on the mixed-materials workload; prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: a 1 m box at 128^3 (dx = 1/128, padded grid 134^3), 8 particles per cell: a von Mises sphere
r = 0.12 (E 2e4, nu 0.45, yield 300 Pa, rho 600), a Drucker-Prager column 0.15 x 0.4 x 0.15 (E 3.5e5,
nu 0.3, 35 deg, rho 1600), a snowball r = 0.08 thrown at (3, 1, 0) m/s (E 1.4e5, nu 0.2, hardening 10,
theta_c 2.5e-2, theta_s 7.5e-3, max hardening 20, rho 400) and one static seeded perturbed icosphere
collider of 5,120 triangles; about 304k particles; synthetic, seeded data.

A step is one substep (dt = 5e-5) of the whole scene with the state resident in HBM (``value``). The
L2 cache (129 MB) is larger than this state, so a 256 MiB buffer is written between timed steps and only
the substeps are timed. ``e2e`` is the same metric through the public solver API with host buffers: one
24 fps frame per step (set_collider_transforms, advance(1/24) at the CFL time step, get_particles and
save_state back to host memory, as the reference's bake runner does every frame).

``--impl reference`` times the CPU implementation of the same substep on all host cores. The reference's
own backend needs warp-lang, which cannot be installed here, so that arm runs the project's C restatement
of the reference kernels (the oracle), labelled as such.

Several GPUs run independent replicas of the scene, one per rank (there is no data exchange in this path).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-substeps/s on 1 GB300, batched vs plain; p50/p99 frame latency"
UNIT = "particle-substeps/s"
DT = 5e-5
FRAME_DT = 1 / 24
G2P_BYTES = 156   # per particle: read x, F, Jp, mat (56 B) + write x, v, C, F, Jp (100 B)
P2G_BYTES = 104   # per particle: read x, v, C, F, Jp, mat
SUBSTEP_BYTES = 204
WORKLOAD = "mixed materials 128^3: von Mises sphere + Drucker-Prager column + snowball + 5120-triangle collider"


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def dist_env():
    from mpm_plugin_gb300.replicas import dist_env as env

    return env()


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs (every 25 ms; only
    the samples whose timestamps fall inside the region count)."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        import datetime

        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)  # the sampler is running before the region starts
        except Exception:
            self.proc = None
        self.t0 = datetime.datetime.now()
        return self

    def __exit__(self, *exc):
        import datetime

        self.t1 = datetime.datetime.now()
        self.out = ""
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        import datetime

        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
                if not (self.t0 <= ts <= self.t1):
                    continue
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _index(device: str) -> int:
    return int(device.split(":")[1]) if ":" in device else 0


def build_scene(device: str = "cuda:0", sample=None):
    """The headline workload (mpm_plugin_gb300.workloads.mixed_scene), its mesh volumes sampled on `device`, or
    by `sample` (the CPU arms pass the oracle's sampler: the same points, no GPU kernel)."""
    from mpm_plugin_gb300.workloads import mixed_scene

    return mixed_scene(res=128, seed=0, device=_index(device), sample=sample)


def _cpu_sampler():
    from oracle import geometry

    return geometry.sample_mesh_volume


def make_gpu_solver(device: str):
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver
    from mpm_plugin_gb300.workloads import add_group

    d, mats, groups, (cv, ct, xf) = build_scene(device)
    s = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device)
    for pos, m, vel in groups:
        add_group(s, pos, m, m, vel)
    s.set_colliders([ColliderGeometry(MeshData(cv, ct), True, 0.5)])
    s.set_collider_transforms(xf[None], xf[None])
    return s, xf


BATCH_FRAME_DT = 1 / 480


def run_batched(device: str, frames: int, n_hi: float = 2e6) -> dict:
    """The batched workload: 64 seeded scenes (n_hi = 2e6: about 24.9M particles, log-uniform 10k-1.7M per
    scene, grids 33^3-176^3; n_hi = 1e5: small scenes of 10k-100k particles), four material models, 0-2
    colliders of 1k-20k triangles, each advancing with its own CFL step. Times `frames` frames of 1/480 s of
    every scene run one at a time through the plain solver, then the same number through one Gb300Batch;
    both after one untimed frame (graph capture, voxel grids)."""
    import torch

    from mpm_plugin_gb300.batch import Gb300Batch
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver
    from mpm_plugin_gb300.workloads import add_group, batched_scenes

    specs = batched_scenes(seed=0, n_hi=n_hi)
    solvers = []
    for d, mats, pos, vel, cols in specs:
        s = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device)
        add_group(s, pos, 0, 0, vel)
        if cols:
            s.set_colliders([ColliderGeometry(MeshData(cv, ct), True, fr) for cv, ct, _, fr in cols])
            xf = np.stack([c[2] for c in cols])
            s.set_collider_transforms(xf, xf)
        solvers.append(s)
    counts = [s.particle_count for s in solvers]

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    from mpm_plugin_gb300 import tune

    # plain: one scene at a time (each scene's frames back to back, as separate bake jobs would run), each
    # with launch choices tuned for it (the autotuner's cache serves scenes of one workload class)
    plain_ps, plain_s, plain_frame_ms, plain_steps = 0.0, 0.0, [], []
    for s, n in zip(solvers, counts):
        st0 = s.advance(BATCH_FRAME_DT)
        snapshot = s.save_state()
        tune.tune_solver(s, st0.dt, BATCH_FRAME_DT, substeps=10)
        s.load_state(snapshot)
        plain_steps.append(st0.substeps)
        for _ in range(frames):
            st, el = timed(lambda: s.advance(BATCH_FRAME_DT))
            plain_ps += n * st.substeps
            plain_s += el
            plain_frame_ms.append(1e3 * el)
    batch = Gb300Batch(solvers)
    tuned = tune.tune_batch(batch, BATCH_FRAME_DT, frames=1)
    batch.advance(BATCH_FRAME_DT)
    launches0 = batch.launch_count()
    batch_ps, batch_s, batch_frame_ms = 0.0, 0.0, []
    for _ in range(frames):
        stats, el = timed(lambda: batch.advance(BATCH_FRAME_DT))
        batch_ps += sum(s.particle_count * st.substeps for s, st in zip(solvers, stats))
        batch_s += el
        batch_frame_ms.append(1e3 * el)
    launches = batch.launch_count() - launches0
    # the batch replays max(steps) substeps a frame; a scene whose own substeps are done idles (its work
    # lists and particle chunks drop out of every kernel): the share of scene-substeps that idle
    last = [st.substeps for st in stats]
    idle_share = 1.0 - sum(last) / (len(last) * max(max(last), 1))
    batch.close()
    for s in solvers:
        s.close()
    plain = plain_ps / plain_s
    batched = batch_ps / batch_s
    return {"value": batched, "plain_value": plain, "unit": UNIT, "ratio": batched / plain,
            "scenes": len(counts), "particles": int(sum(counts)), "frames": frames, "frame_dt": BATCH_FRAME_DT,
            "batch_frame_ms": {"p50": float(np.percentile(batch_frame_ms, 50)),
                               "p99": float(np.percentile(batch_frame_ms, 99))},
            "plain_scene_frame_ms": {"p50": float(np.percentile(plain_frame_ms, 50)),
                                     "p99": float(np.percentile(plain_frame_ms, 99))},
            "gpu_launches_per_frame": launches / frames, "tuned": tuned,
            "substeps_per_frame": {"min": int(min(last)), "max": int(max(last))},
            "idle_scene_substep_share": idle_share,
            "timing": "host clock around advance calls with device synchronisation; state resident in HBM"}


class _FrameSink:
    """Stands in for the cache writer: receives every frame (positions, velocities) and counts the bytes."""

    def __init__(self):
        self.bytes = 0

    def write_frame(self, frame, particles):
        self.bytes += particles.positions.nbytes + particles.velocities.nbytes


def serve_trace(seconds: float, rate: float, seed: int = 0, frames: int = 8, res: int = 128):
    """Poisson arrivals (mean `rate` per second) over `seconds`; each request one seeded pour job of `frames`
    frames at resolution `res`."""
    from mpm_plugin_gb300.serve import BakeJob
    from mpm_plugin_gb300.workloads import pour_job as pour_job_spec

    rng = np.random.default_rng(seed)
    t, trace, i = 0.0, [], 0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > seconds:
            return trace
        d, mats, setup, before, nf, fps, max_n, tris = pour_job_spec(seed * 1000 + i, res=res, frames=frames,
                                                                     side_range=(0.25, 0.45))
        trace.append((t, BakeJob(f"job{i}", d, mats, nf, fps, setup=setup, before_frame=before,
                                 writer=_FrameSink(), max_particles=max_n, collider_triangles=tris)))
        i += 1


def run_serving(device: str, seconds: float, rate: float = 3.0, budget_gb: float = 6.0, frames: int = 8) -> dict:
    """Serving: a Poisson trace of pour jobs (128^3, a pile of 130k-760k particles plus a 2 m/s disc inflow, a
    2,048-triangle torus turning at 1 rev/s, `frames` frames at 24 fps each) served by the bake server with an
    admission budget of `budget_gb` (a few jobs' worth, so admission waits on memory), against the same trace
    served sequentially by the plain solver (each job alone, in arrival order, starting when it has arrived
    and the one before has finished). The metric's trace (8M-particle pours, 48 frames, 4 per second for 10
    minutes, 150 GB) is two orders of magnitude beyond one GPU; this one keeps its shape: Poisson arrivals at
    about the GPU's capacity, so queues form, with memory the binding limit on admission."""
    import torch

    from mpm_plugin_gb300.serve import BakeServer
    from mpm_plugin_gb300.solver import Gb300Solver

    trace = serve_trace(seconds, rate, frames=frames)
    srv = BakeServer(int(budget_gb * (1 << 30)), device=device)
    rep = srv.run(trace)
    srv.close()
    served = rep.summary()

    # the same trace, sequentially through the plain solver
    trace = serve_trace(seconds, rate, frames=frames)
    clock, frame_ms, job_s, ps = 0.0, [], [], 0.0
    for arrival, job in trace:
        clock = max(clock, arrival)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = Gb300Solver(job.domain, job.materials, job.gravity, job.particles_per_cell, device=device)
        job.setup(s)
        last = time.perf_counter()
        for k in range(1, job.frames + 1):
            job.before_frame(s, k)
            n = s.particle_count
            st = s.advance(1.0 / job.fps)
            ps += n * st.substeps
            job.writer.write_frame(k, s.get_particles())
            now = time.perf_counter()
            frame_ms.append(1e3 * (now - last))
            last = now
        s.close()
        clock += time.perf_counter() - t0
        job_s.append(clock - arrival)
    plain = {"frame_latency_ms": {"p50": float(np.percentile(frame_ms, 50)), "p99": float(np.percentile(frame_ms, 99))},
             "job_latency_s": {"p50": float(np.percentile(job_s, 50)), "p99": float(np.percentile(job_s, 99))},
             "particle_substeps_per_s": ps / clock}
    jl = list(rep.job_latency_s.values())
    served["job_latency_s"] = {"p50": float(np.percentile(jl, 50)), "p99": float(np.percentile(jl, 99))}
    return {"requests": len(trace), "rate_per_s": rate, "seconds": seconds, "budget_gb": budget_gb,
            "served": served, "plain_sequential": plain,
            "ratio": served["particle_substeps_per_s"] / plain["particle_substeps_per_s"],
            "frames_per_job": frames,
            "workload": f"Poisson pour jobs, 128^3, {frames} frames at 24 fps, inflow + rotating 2,048-triangle torus; "
                        "frames handed to an in-memory sink in place of the cache writer"}


def large_scene(res: int, pile_top: float, seed: int = 3):
    from mpm_plugin_gb300.workloads import large_scene as make

    return make(res, pile_top, seed)


def run_large(device: str, frames: int, fp64_mode: int = 0, tuned_cfg: dict | None = None) -> dict:
    """The 256^3 inflow workload (about 7.5M particles at the start), driven as the bake runner drives it:
    per 24 fps frame, four pieces of 1/96 s, each with the collider's start and end pose, an advance at the
    CFL step and an emission (occupancy query + add_particles); then the frame's particles are read back.
    One untimed frame first, then the autotuner (unless tuned_cfg is given). FP64 conservation totals are read
    at the start and the end. fp64_mode: the
    Drucker-Prager return mapping redone in FP64 for marginal decisions (1) or not (0)."""
    import torch

    from mpm_plugin_gb300 import _abi, tune
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver

    dev = _index(device)
    d, mats, pile, (tv, tt), pose, emit = large_scene(256, 0.155)
    s = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device)
    s.add_particles(pile, np.zeros_like(pile), np.zeros(len(pile), np.int32), np.zeros(len(pile), np.int32))
    s.set_colliders([ColliderGeometry(MeshData(tv, tt), True, 0.4)])
    s.set_collider_transforms(pose(0.0)[None], pose(0.0)[None])
    if tuned_cfg is not None:  # the FP64 run keeps the FP32 run's launch choices
        tune.apply(s, tuned_cfg, tune.gpu_key(device)[1], solver=True)
        tuned = {**tuned_cfg, "cached": True}
    s.set_option(_abi.OPT_FP64_CLAMP, fp64_mode)
    n0 = s.particle_count
    c0 = s.conservation()
    t_adv = t_emit = t_read = 0.0
    ps, substeps, emitted, frame_ms = 0.0, 0, 0, []
    for f in range(frames + 1):
        if f == 1 and tuned_cfg is None:
            # launch choices tuned on the scene after the untimed frame: the inflow has begun appending
            # particles out of grid order, which the pile's initial lattice order does not show
            tuned = tune.tune_solver(s, 8e-5, 1 / 96, substeps=100)
        f0 = time.perf_counter()
        fa = fe = 0.0
        for piece in range(4):
            k = 4 * f + piece
            s.set_collider_transforms(pose(k / 96)[None], pose((k + 1) / 96)[None])
            n = s.particle_count
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = s.advance(1 / 96)
            t1 = time.perf_counter()
            added = emit(s, k, dev)
            t2 = time.perf_counter()
            if f > 0:
                ps += n * st.substeps
                substeps += st.substeps
                emitted += added
                fa += t1 - t0
                fe += t2 - t1
        t3 = time.perf_counter()
        s.get_particles()
        t4 = time.perf_counter()
        if f > 0:
            t_adv += fa
            t_emit += fe
            t_read += t4 - t3
            frame_ms.append(1e3 * (t4 - f0))
    c1 = s.conservation()
    n1 = s.particle_count
    redo = s.fp64_redo_lanes()
    # kernel-group times of a few substeps at the end state (event nodes in the substep graph)
    s.set_option(_abi.OPT_KERNEL_TIMING, 1)
    s.kernel_times(reset=True)
    for _ in range(4):
        s.substep(8e-5, 1.0, 1 / 96)
    kt = s.kernel_times(reset=True)
    s.set_option(_abi.OPT_KERNEL_TIMING, 0)
    final = s.save_state() if fp64_mode == 0 else None
    pose_end = pose((4 * frames + 4) / 96)
    s.close()
    total = t_adv + t_emit + t_read
    out = {"value": ps / total, "advance_only": ps / t_adv, "unit": UNIT, "frames": frames,
           "fp64_return_mapping": {0: "off (FP32; FP64 only for SVDs that did not converge)",
                                   1: "marginal decisions redone in FP64"}[fp64_mode],
           "fp64_redo_lanes": redo, "fp64_redo_share": redo / max(ps, 1.0),
           "particles_start": n0, "particles_end": n1, "emitted": emitted, "substeps": substeps,
           "seconds": {"advance": t_adv, "emission": t_emit, "read_back": t_read},
           "frame_ms": {"p50": float(np.percentile(frame_ms, 50)), "p99": float(np.percentile(frame_ms, 99))},
           "tuned": tuned,
           "kernels_ms_per_substep": {k: t / max(c, 1) for k, (t, c) in kt.items()},
           "conservation_fp64": {"mass": [c0["mass"], c1["mass"]], "ke": [c0["ke"], c1["ke"]],
                                 "momentum_z": [float(c0["momentum"][2]), float(c1["momentum"][2])]}}
    return out, final, (tv, tt), pose_end


def fp64_subbox_error(device: str, state: dict, torus_mesh, pose, seed: int = 7, checks=(100, 200, 300),
                      dt: float = 5e-5) -> dict:
    """Error against the FP64 oracle on a seeded sub-box of the pour: the particles of the large workload's
    final state inside an 8 cm cube at a seeded place on the pile floor, in a 25 cm domain around it at the
    same dx (walls at its sides and floor), with the torus at its final pose. The same substeps on the GPU
    (FP32 bulk, marginal return-mapping decisions in FP64) and on the FP64 oracle (the checker); relative
    errors of x, v, F and of the invariants after every 100 substeps, and with the FP64 redo off at the end."""
    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.interface import ColliderGeometry, MaterialParams, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver
    from mpm_plugin_gb300.workloads import make_domain
    from oracle.oracle import OracleSolver

    rng = np.random.default_rng(seed)
    cx, cy = (float(c) for c in rng.uniform(0.3, 0.7, 2))
    x = state["x"]
    sel = (np.abs(x[:, 0] - cx) <= 0.04) & (np.abs(x[:, 1] - cy) <= 0.04) & (x[:, 2] <= 0.08)
    sub = {k: np.ascontiguousarray(v[sel]) for k, v in state.items()}
    d = make_domain(64, (cx - 0.125, cy - 0.125, 0.0), (cx + 0.125, cy + 0.125, 0.25))
    mats = [MaterialParams("pour", "drucker_prager", 3.5e5, 0.3, 1600.0, friction_angle_deg=30.0)]
    tv, tt = torus_mesh
    xf = pose.astype(np.float32)[None]
    gs = [Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device) for _ in range(2)]
    gs[0].set_option(_abi.OPT_FP64_CLAMP, 1)
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f64", threads=os.cpu_count() or 1)
    for g in gs:
        g.load_state(sub)
        g.set_colliders([ColliderGeometry(MeshData(tv, tt), True, 0.4)])
        g.set_collider_transforms(xf, xf)
    o.load_state(sub)
    o.set_colliders([(tv, tt, True, 0.4)])
    o.set_collider_transforms(xf, xf)
    steps = max(checks)
    o.frame_dt = steps * dt
    pm = float(np.float32(1600.0) * np.float32((0.25 / 64) ** 3 / 8))
    rel = lambda u, w: float(np.linalg.norm(u - w) / max(np.linalg.norm(w), 1e-30))  # noqa: E731

    def errors(a, b):
        va, vb = a["v"].astype(np.float64), b["v"].astype(np.float64)
        return {"x": rel(a["x"], b["x"]), "v": rel(a["v"], b["v"]), "F": rel(a["F"], b["F"]),
                "momentum": rel((pm * va).sum(0), (pm * vb).sum(0)),
                "com": rel(a["x"].astype(np.float64).mean(0), b["x"].astype(np.float64).mean(0)),
                "ke": abs((va * va).sum() - (vb * vb).sum()) / max((vb * vb).sum(), 1e-30)}

    t0 = time.perf_counter()
    per = {}
    for k in range(steps):
        sk = (k + 1) / steps
        for g in gs:
            g.substep(dt, sk, steps * dt)
        o.substep(dt, sk)
        if k + 1 in checks:
            per[k + 1] = errors(gs[0].save_state(), o.save_state())
    off = errors(gs[1].save_state(), o.save_state())
    redo = gs[0].fp64_redo_lanes()
    for g in gs:
        g.close()
    return {"particles": int(sel.sum()), "sub_box": [[cx - 0.04, cy - 0.04, 0.0], [cx + 0.04, cy + 0.04, 0.08]],
            "dt": dt, "errors_every_100_substeps": per, f"errors_at_{steps}_fp64_off": off,
            "fp64_redo_lanes": redo, "oracle_seconds": time.perf_counter() - t0,
            "reference": "FP64 oracle (C restatement of the reference kernels, REAL = double)"}


def run_surface(device: str, repeats: int = 3) -> dict:
    """Surfacing (mpm_plugin_gb300.surface, the drop-in for mpm_surface/field.py) of two particle sets with
    the default settings (detail 1, smoothing 2, iso 0.35): the 256^3 pour's pile (7.45M particles at the
    8-per-cell spacing dx / 2) and a seeded Gaussian blob of 1M particles at spacing 0.004. Each call is timed
    end to end through surface_particles (host set-up, copies in, splat, normalisation, marching cubes,
    vertex velocities, copies out), median of `repeats` after one untimed call. The CPU restatement's splat
    alone (oracle.surface, float64 numpy per particle) is timed on 2,000 particles of the blob beside it."""
    import torch

    from mpm_plugin_gb300.surface import SurfaceSettings, surface_particles
    from oracle import surface as S

    from mpm_plugin_gb300.workloads import cell_size

    d, _, pile, _, _, _ = large_scene(256, 0.155)
    rng = np.random.default_rng(5)
    sets = {"pour_pile_256": (pile.astype(np.float32), rng.normal(0, 0.1, pile.shape).astype(np.float32),
                              cell_size(d) / 2),
            "blob_1m": ((rng.normal(0, 0.05, (1_000_000, 3)) + 0.5).astype(np.float32),
                        rng.normal(0, 1.0, (1_000_000, 3)).astype(np.float32), 0.004)}
    out = {}
    for name, (x, v, spacing) in sets.items():
        st = SurfaceSettings()
        surface_particles(x, v, spacing, st, device=device)
        ts = []
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mesh = surface_particles(x, v, spacing, st, device=device)
            ts.append(time.perf_counter() - t0)
        t = float(np.median(ts))
        cell = spacing / st.detail
        pad = 2.0 * spacing * st.smoothing + 2.0 * cell
        dims = [int(np.ceil(e / cell)) + 1 for e in x.max(0) + pad - (x.min(0).astype(np.float64) - pad)]
        out[name] = {"particles": len(x), "field_nodes": int(np.prod(dims)), "verts": len(mesh.verts),
                     "tris": len(mesh.tris), "ms": 1e3 * t, "particles_per_s": len(x) / t}
    x, v, spacing = sets["blob_1m"]
    sample = x[:2000]
    origin, dims, cell, h = S.grid_params(x, spacing, 1.0, 2.0)
    t0 = time.perf_counter()
    S.splat(sample, v[:2000], np.float32(origin), np.float32(1.0 / cell), np.float32(cell), np.float32(h), dims)
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": len(sample) / el, "unit": "particles/s (splat only)", "cores": 1,
                           "kind": "port", "sample": f"{len(sample)} particles of blob_1m, {el:.1f} s"}
    return out


def run_small(device: str, substeps: int = 1000, cpu_substeps: int = 50) -> dict:
    """The small plain workload: a fixed-corotated jelly cube of side 0.25 centred at (0.5, 0.6, 0.5) in a
    1 m box at 64^3, 8 particles per cell from a seeded stratified jitter (32,768 particles), E 1e5, nu 0.3,
    rho 1000, at rest, dt 1e-4, `substeps` substeps through the fixed-dt entry (advance(1e-4) takes exactly
    one substep at this dt, under the CFL limit). The reference's single wall friction applies to all walls
    (its sticky-floor / slip-wall split is not expressible there). The FP32 oracle is timed on the first
    `cpu_substeps` substeps of the same scene on all host cores."""
    import torch

    from mpm_plugin_gb300.solver import Gb300Solver
    from mpm_plugin_gb300.workloads import jelly_cube
    from oracle.oracle import OracleSolver

    d, mats, pos = jelly_cube(64)
    z = np.zeros(len(pos), np.int32)
    from mpm_plugin_gb300 import tune

    g = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device)
    g.add_particles(pos, np.zeros_like(pos), z, z)
    # launch choices timed as this workload runs (run_substeps of `substeps`; shorter windows picked a
    # configuration 10 % slower than the best, measured)
    tuned = tune.tune_solver(g, 1e-4, 1e-4, substeps=substeps, runs=True)
    g.run_substeps(1e-4, 10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.run_substeps(1e-4, substeps)  # one call, the captured substep graph replayed `substeps` times
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    g.close()
    threads = os.cpu_count() or 1
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=threads)
    o.add_particles(pos, np.zeros_like(pos), z, z)
    o.frame_dt = 1e-4
    t0 = time.perf_counter()
    for _ in range(cpu_substeps):
        o.substep(1e-4, 1.0)
    cpu_s = time.perf_counter() - t0
    n = len(pos)
    return {"value": n * substeps / gpu_s, "unit": UNIT, "particles": n, "substeps": substeps,
            "ms_per_substep": 1e3 * gpu_s / substeps,
            "timing": "host clock around one run_substeps call with device synchronisation (launch-bound at this "
                      "size: about 7 kernels per substep)",
            "tuned": tuned,
            "cpu_baseline": {"value": n * cpu_substeps / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{cpu_substeps} substeps of the same scene"}}


def cpu_oracle_time(threads: int, budget_s: float):
    """FP32 oracle (C restatement of the reference kernels, OpenMP) on the same scene; returns rate, sample."""
    from mpm_plugin_gb300.workloads import add_group
    from oracle.oracle import OracleSolver

    d, mats, groups, (cv, ct, xf) = build_scene(sample=_cpu_sampler())
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=threads)
    for pos, m, vel in groups:
        add_group(o, pos, m, m, vel)
    o.set_colliders([(cv, ct, True, 0.5)])
    o.set_collider_transforms(xf[None], xf[None])
    n = o.particle_count
    o.substep(DT, 1.0)  # warm-up
    t0 = time.perf_counter()
    o.substep(DT, 1.0)
    t1 = time.perf_counter() - t0
    k = max(1, min(200, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(k):
        o.substep(DT, 1.0)
    el = time.perf_counter() - t0
    return n * k / el, n, k, el


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from mpm_plugin_gb300.workloads import add_group
    from oracle.oracle import OracleSolver

    d, mats, groups, (cv, ct, xf) = build_scene(sample=_cpu_sampler())
    o = OracleSolver(d, mats, (0.0, 0.0, -9.81), 8, precision="f32", threads=threads)
    for pos, m, vel in groups:
        add_group(o, pos, m, m, vel)
    o.set_colliders([(cv, ct, True, 0.5)])
    o.set_collider_transforms(xf[None], xf[None])
    n = o.particle_count
    for _ in range(args.warmup):
        o.substep(DT, 1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.substep(DT, 1.0)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": n, "grid": 128, "dt": DT},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} substeps of the full {n}-particle scene on {threads} threads; "
                                       "the reference's Warp backend cannot be installed (no warp-lang), so this "
                                       "is the C restatement of its kernels"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, world, rank, local):
    import torch

    device = f"cuda:{local}"
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(device))
    from mpm_plugin_gb300 import _abi

    solver, xf = make_gpu_solver(device)
    n = solver.particle_count
    stream = torch.cuda.ExternalStream(solver.stream, device=device)  # the flush runs on the solver's stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)

    from mpm_plugin_gb300 import tune

    tuned = tune.tune_solver(solver, DT, FRAME_DT, substeps=50)  # launch choices for this GPU and workload
    for _ in range(args.warmup):
        solver.substep(DT, 1.0, FRAME_DT)
    solver.synchronize()

    # timed region: K substeps, L2 written between them. Each substep replays its captured graph with CUDA
    # events recorded at the graph's two ends on the solver's stream (MPM_OPT_KERNEL_TIMING 2); the value is
    # the sum of those substep times, so the writes between substeps are not in it.
    def timed_substeps(mode, clocks=None):
        """K substeps under kernel timing `mode`; returns the kernels they launched."""
        solver.set_option(_abi.OPT_KERNEL_TIMING, mode)
        solver.substep(DT, 1.0, FRAME_DT)  # capture the timed graph outside the timed region
        solver.kernel_times(reset=True)
        solver.substep_times(reset=True)
        launches0 = solver.launch_count()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.__enter__()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(float(k))
                solver.substep(DT, 1.0, FRAME_DT)
        torch.cuda.synchronize()
        if clocks:
            clocks.__exit__(None, None, None)
        if world > 1:
            torch.distributed.barrier()
        return solver.launch_count() - launches0

    clk = Clocks(local)
    launches = timed_substeps(2, clk)
    total_ms, _ = solver.substep_times(reset=True)
    # the same substeps with events between the kernel groups (which also break the launch chain there): the
    # per-kernel times of the breakdown and the roofline
    timed_substeps(1)
    ktimes = solver.kernel_times(reset=True)

    # the same timed substeps in deterministic mode (fixed-point P2G), with launch choices tuned for it
    solver.set_option(_abi.OPT_DETERMINISTIC, 1)
    det_tuned = tune.tune_solver(solver, DT, FRAME_DT, substeps=50, deterministic=True)
    for _ in range(3):
        solver.substep(DT, 1.0, FRAME_DT)
    timed_substeps(2)
    det_ms, _ = solver.substep_times(reset=True)
    timed_substeps(1)
    det_times = solver.kernel_times(reset=True)
    solver.set_option(_abi.OPT_DETERMINISTIC, 0)
    solver.set_option(_abi.OPT_KERNEL_TIMING, 0)

    # end to end through the solver API: one bake frame per step, host buffers, on a fresh copy of the scene
    # (the frames then cover the same stretch of the simulation whatever --steps was)
    fp64_lanes = solver.fp64_lanes()
    solver.close()
    solver, xf = make_gpu_solver(device)
    tune.tune_solver(solver, DT, FRAME_DT, substeps=50)  # the cached choice
    e2e_frames, frame_ms, substeps = max(2, args.e2e_frames), [], 0
    h2d = 2 * 64  # the collider's start and end world matrices
    d2h = n * (12 + 12 + 36 + 36 + 4 + 4 + 4)  # the full state (x v C F Jp mat emitter) covers get_particles too
    solver.advance(FRAME_DT)  # warm the CFL path and the graph
    solver.read_begin(("x", "v", "C", "F", "Jp", "mat", "emitter")).wait()
    # As the bake runner does per frame (transforms, advance, particles for the cache, state for the checkpoint)
    # but with the frame's read-back overlapping the next frame's substeps: read_begin right after an advance,
    # wait for it once the next advance has run (the state read covers get_particles' arrays too).
    pending = None
    for _ in range(e2e_frames):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.set_collider_transforms(xf[None], xf[None])
        st = solver.advance(FRAME_DT)
        if pending is not None:
            pending.wait()
        pending = solver.read_begin(("x", "v", "C", "F", "Jp", "mat", "emitter"))
        frame_ms.append(1e3 * (time.perf_counter() - t0))
        substeps += st.substeps
    t0 = time.perf_counter()
    pending.wait()
    frame_ms[-1] += 1e3 * (time.perf_counter() - t0)
    e2e = n * substeps / (sum(frame_ms) / 1e3)
    # where a late frame's substeps go (outside the timed frames): kernel-group events over 20 substeps at the
    # state the frames left, with the collider contact the early substeps of the headline do not have
    solver.set_option(_abi.OPT_KERNEL_TIMING, 1)
    solver.kernel_times(reset=True)
    for _ in range(20):
        solver.substep(DT, 1.0, FRAME_DT)
    late = solver.kernel_times(reset=True)
    solver.set_option(_abi.OPT_KERNEL_TIMING, 0)
    late_ms = {k: late[k][0] / max(late[k][1], 1) for k in late}

    from mpm_plugin_gb300.replicas import reduce_timing

    total_s, units = reduce_timing(total_ms / 1e3, float(n) * args.steps, device)  # slowest rank, all ranks' units
    e2e_s, e2e_units = reduce_timing(sum(frame_ms) / 1e3, float(n) * substeps, device)
    if rank != 0:
        return
    total_ms = 1e3 * total_s
    value = units / total_s
    e2e_all = e2e_units / e2e_s

    names = {"p2g": P2G_BYTES, "g2p": G2P_BYTES}
    # The roofline kernel is G2P, the one the substep's HBM target is stated for; P2G, which takes about as
    # long (the two swap places between runs), is reported beside it under particle_kernels.
    dom = "g2p"
    avg_ms = {k: (ktimes[k][0] / max(ktimes[k][1], 1)) for k in ktimes}
    peak, peak_kind = peaks()
    bytes_per_launch = names[dom] * n
    achieved = bytes_per_launch / (avg_ms[dom] / 1e3) / 1e9
    tdoc = {}
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            tdoc = json.loads(tfile.read_text())
        except ValueError:
            tdoc = {}
    traffic, warp_inst = tdoc.get(dom), tdoc.get(f"{dom}_warp_instructions")
    clocks = clk.summary()
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0

    def issue_frac_of(k):
        """The kernel's warp instructions (ncu, committed) over what 4 schedulers per SM issue in its time."""
        inst = tdoc.get(f"{k}_warp_instructions")
        return inst / (sms * 4 * mhz * 1e6 * avg_ms[k] / 1e3) if inst else None

    issue_frac = issue_frac_of(dom)
    particle_kernels = {k: {"algorithmic_bytes_per_launch": names[k] * n, "ms_per_launch": avg_ms[k],
                            "achieved_gbs": names[k] * n / (avg_ms[k] / 1e3) / 1e9,
                            "frac": names[k] * n / (avg_ms[k] / 1e3) / 1e9 / peak,
                            "traffic": tdoc.get(k), "issue_frac": issue_frac_of(k)} for k in ("p2g", "g2p")}
    cpu_rate, cpu_n, cpu_k, cpu_el = cpu_oracle_time(os.cpu_count() or 1, args.cpu_budget)
    batched = None
    if args.batched_frames > 0:
        solver.close()
        batched = run_batched(device, args.batched_frames)
        batched["small_scenes"] = run_batched(device, args.batched_frames, n_hi=1e5)
    serving = (run_serving(device, args.serve_seconds, args.serve_rate, args.serve_budget_gb, args.serve_frames)
               if args.serve_seconds > 0 else None)
    large = None
    if args.large_frames > 0:
        large, final, tmesh, pose_end = run_large(device, args.large_frames)
        on = run_large(device, args.large_frames, fp64_mode=1, tuned_cfg=large["tuned"])[0]
        large["fp64_on"] = {k: on[k] for k in ("value", "advance_only", "fp64_return_mapping", "fp64_redo_lanes",
                                                "fp64_redo_share", "substeps", "kernels_ms_per_substep")}
        large["fp64_oracle_error"] = fp64_subbox_error(device, final, tmesh, pose_end)
    small = run_small(device) if args.small else None
    surface = run_surface(device) if args.surface and rank == 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "particles": n, "grid": 128, "dt": DT, "parallelism": f"replicas{world}",
                   "l2": "256 MiB written between timed substeps (state is smaller than L2)",
                   "timing": "CUDA events at the two ends of each substep's graph on the solver's stream, summed "
                             "over the timed substeps; the L2 writes between them are outside"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": dom, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": bytes_per_launch,
                     "issue_frac": issue_frac, "warp_instructions_per_launch": warp_inst,
                     "particle_kernels": particle_kernels,
                     "note": "HBM fraction of the algorithmic bytes; the kernel is bound by instruction issue and "
                             "latency (issue_frac: warp instructions / (SMs x 4 x SM clock x kernel time))"},
        "kernels_ms_per_launch": avg_ms,
        "substep_bytes": {"algorithmic_per_particle": SUBSTEP_BYTES,
                          "achieved_gbs": SUBSTEP_BYTES * n * args.steps / (total_ms / 1e3) / 1e9},
        "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{cpu_k} substeps of the full {cpu_n}-particle scene, {cpu_el:.1f} s"},
        "e2e": {"value": e2e_all, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "step": "one 24 fps frame via the solver API (transforms, advance, full state read back; each "
                        "frame's read-back overlaps the next frame's substeps), frames 2-5 of a fresh copy of "
                        "the scene",
                "substeps_per_frame": substeps / e2e_frames,
                "late_frame_kernels_ms_per_substep": late_ms},
        "frame_latency_ms": {"p50": float(np.percentile(frame_ms, 50)), "p99": float(np.percentile(frame_ms, 99))},
        "gpu_launches": launches,
        "clocks": clocks,
        "fp64_svd_lanes": fp64_lanes,
        "tuned": tuned,
        "deterministic": {"value": n * args.steps / (det_ms / 1e3), "unit": UNIT,
                          "kernels_ms_per_launch": {k: t / max(c, 1) for k, (t, c) in det_times.items()},
                          "tuned": det_tuned},
        "batched": batched,
        "serving": serving,
        "large": large,
        "small": small,
        "surface": surface,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_profile_case(args) -> None:
    """A fixed case for profilers (no timing, no output but one line): `--profile-case mix128` (the headline
    scene), `mix128_late` (the same scene after five 24 fps frames through the solver API, the snowball and
    the column pressing on the collider; only its profiled substeps run between cudaProfilerStart and
    cudaProfilerStop, for `ncu --profile-from-start off`) or `pour256` (the large workload's 7.45M-particle
    pile and torus, no inflow), with the given launch choices, `--profile-substeps` explicit substeps without
    graphs, so each kernel is its own launch and a profiler can select launches by kernel name and count."""
    import torch
    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
    from mpm_plugin_gb300.solver import Gb300Solver

    device = "cuda:0"
    if args.profile_case in ("mix128", "mix128_late"):
        s, xf = make_gpu_solver(device)
        dt = DT
        if args.profile_case == "mix128_late":
            for _ in range(5):
                s.set_collider_transforms(xf[None], xf[None])
                s.advance(FRAME_DT)
    else:
        d, mats, pile, (tv, tt), pose, _ = large_scene(256, 0.155)
        s = Gb300Solver(d, mats, (0.0, 0.0, -9.81), 8, device=device)
        z = np.zeros(len(pile), np.int32)
        s.add_particles(pile, np.zeros_like(pile), z, z)
        s.set_colliders([ColliderGeometry(MeshData(tv, tt), True, 0.4)])
        s.set_collider_transforms(pose(0.0)[None], pose(1 / 96)[None])
        dt = 8e-5
    s.set_option(_abi.OPT_USE_GRAPH, 0)
    s.set_option(_abi.OPT_G2P_VARIANT, args.g2p_variant)
    s.set_option(_abi.OPT_SORT_INTERVAL, args.sort_interval)
    s.set_option(_abi.OPT_BLOCK_SWEEP, args.block_sweep)
    s.set_option(_abi.OPT_P2G_TILE, args.p2g_tile)
    s.set_option(_abi.OPT_P2G_GROUP, args.p2g_group)
    s.set_option(_abi.OPT_P2G_MERGE, args.p2g_merge)
    s.set_option(_abi.OPT_DETERMINISTIC, args.deterministic)
    s.set_option(_abi.OPT_FP64_CLAMP, args.fp64_clamp)
    late = args.profile_case == "mix128_late"
    if late:
        s.synchronize()
        torch.cuda.profiler.start()
    for k in range(args.profile_substeps):
        s.substep(dt, (k + 1) / args.profile_substeps, 1 / 96)
    s.synchronize()
    if late:
        torch.cuda.profiler.stop()
    print(f"profile case {args.profile_case}: {s.particle_count} particles, {args.profile_substeps} substeps")
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline work")
    ap.add_argument("--e2e-frames", type=int, default=4, help="24 fps frames timed through the solver API")
    ap.add_argument("--small", type=int, default=1, help="measure the 32k-particle jelly workload (0: skip)")
    ap.add_argument("--large-frames", type=int, default=1,
                    help="24 fps frames of the 256^3 inflow workload (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=120.0,
                    help="seconds of Poisson bake requests for the serving measurement (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=3.0, help="bake requests per second")
    ap.add_argument("--serve-frames", type=int, default=8, help="frames per bake request")
    ap.add_argument("--serve-budget-gb", type=float, default=6.0, help="admission budget of the bake server")
    ap.add_argument("--batched-frames", type=int, default=3,
                    help="frames of the 64-scene batched workload, plain and batched (0: skip)")
    ap.add_argument("--surface", type=int, default=1, help="measure the surfacer (0: skip)")
    ap.add_argument("--profile-case", choices=["mix128", "mix128_late", "pour256"], default=None,
                    help="run a fixed case for a profiler instead of the benchmark (see run_profile_case)")
    ap.add_argument("--profile-substeps", type=int, default=30)
    ap.add_argument("--g2p-variant", type=int, default=0)
    ap.add_argument("--sort-interval", type=int, default=0)
    ap.add_argument("--block-sweep", type=int, default=0)
    ap.add_argument("--p2g-tile", type=int, default=0)
    ap.add_argument("--p2g-group", type=int, default=32)
    ap.add_argument("--p2g-merge", type=int, default=1)
    ap.add_argument("--deterministic", type=int, default=0, help="profiling case in deterministic mode")
    ap.add_argument("--fp64-clamp", type=int, default=0)
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()

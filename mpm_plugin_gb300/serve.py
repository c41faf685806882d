"""Bake server: continuous batching of bake jobs on one GPU under a device-memory budget.

The reference bakes one scene per process, frame by frame (mpm_core/bake.py:195-213): per frame it sets the
collider transforms, advances, emits, reads the particles back and hands them to the cache writer. The
server keeps that per-job contract for many jobs at once:

* jobs arrive on a trace and wait in FIFO order; a job is admitted when its estimated device footprint fits
  in the budget beside the jobs already resident (a job larger than the whole budget is rejected);
* admitted jobs join one Gb300Batch and stay resident (particles, grid, colliders in HBM) until their last
  frame; every tick advances every resident job by one of its frames in one batched launch sequence, so jobs
  that arrive while others run overlap with them on the device;
* each finished frame is read back and handed to the job's writer (``write_frame(frame, ParticleData)``,
  the interface of mpm_core.cache.CacheWriter) on a writer thread, off the simulation's critical path;
* per-frame latency (time between a job's consecutive frames, the first one counted from admission), job
  latency (arrival to last frame written) and aggregate particle-substeps/s are recorded.
"""

from __future__ import annotations

import math
import queue
import threading
import time
from collections import deque
from collections.abc import Callable
from dataclasses import dataclass, field

import numpy as np

from mpm_plugin_gb300.interface import ParticleData, domain_grid_dims

PARTICLE_BYTES = 152  # arena words per particle x 4 B (x v C F Jp stress mat emitter id, SVD basis)


@dataclass
class BakeJob:
    """One bake: a scene, a frame count and what happens around each frame.

    setup(solver) adds the initial particles and colliders; before_frame(solver, k) runs before frame k
    (1-based) is advanced (collider transforms, emission); writer.write_frame(k, particles) receives each
    frame. max_particles bounds the particle count (emission included) for the footprint estimate.
    """

    name: str
    domain: object
    materials: list
    frames: int
    fps: float = 24.0
    gravity: tuple = (0.0, 0.0, -9.81)
    particles_per_cell: int = 8
    setup: Callable | None = None
    before_frame: Callable | None = None
    writer: object | None = None
    max_particles: int = 0
    collider_triangles: int = 0


def estimate_device_bytes(domain, max_particles: int, collider_triangles: int = 0) -> int:
    """Upper estimate of a job's device memory: two particle arenas plus per-particle sort, removal and
    candidate scratch, the padded blocked grid with its work lists and occupancy scratch, and the colliders'
    BVHs and narrow-band voxel grids (3.0 KB per triangle for the mixed workload's 5,120-triangle sphere,
    5.0 KB for the pour's 20,480-triangle torus; 6 KB counted). Capacity doubles on growth, so particles
    count twice."""
    dims = domain_grid_dims(domain)
    nodes = math.prod(-(-d // 4) * 4 for d in dims)
    cap = 2 * max(int(max_particles), 4096)
    per_particle = 2 * PARTICLE_BYTES + 12 + 16 + 4 + 72
    per_node = 16 + 4 + 4 + 8 + 1
    return cap * per_particle + nodes * per_node + collider_triangles * (128 + 16 + 6144) + (8 << 20)


@dataclass
class _Run:
    job: BakeJob
    solver: object
    reserved: int
    arrival: float
    admitted: float
    frame: int = 0
    last: float = 0.0


@dataclass
class ServeReport:
    frame_latency_ms: list = field(default_factory=list)
    job_latency_s: dict = field(default_factory=dict)
    rejected: list = field(default_factory=list)
    failed: dict = field(default_factory=dict)
    particle_substeps: float = 0.0
    busy_s: float = 0.0
    wall_s: float = 0.0
    max_resident: int = 0
    max_reserved: int = 0
    admit_wait_s: list = field(default_factory=list)  # per admitted job: admission time - arrival
    max_queue: int = 0                                 # most jobs that had arrived and waited for admission

    def summary(self) -> dict:
        lat = self.frame_latency_ms
        return {"frames": len(lat),
                "frame_latency_ms": {"p50": float(np.percentile(lat, 50)) if lat else None,
                                     "p99": float(np.percentile(lat, 99)) if lat else None},
                "jobs": len(self.job_latency_s), "rejected": len(self.rejected), "failed": len(self.failed),
                "particle_substeps_per_s": self.particle_substeps / self.wall_s if self.wall_s else 0.0,
                "busy_particle_substeps_per_s": self.particle_substeps / self.busy_s if self.busy_s else 0.0,
                "max_resident_jobs": self.max_resident, "max_reserved_bytes": self.max_reserved,
                "admission_wait_s": {"p50": float(np.percentile(self.admit_wait_s, 50)) if self.admit_wait_s else None,
                                     "p99": float(np.percentile(self.admit_wait_s, 99)) if self.admit_wait_s else None,
                                     "max": float(max(self.admit_wait_s)) if self.admit_wait_s else None},
                "max_queue": self.max_queue}


class _Writer(threading.Thread):
    """Runs write callbacks in order on one thread, so the simulation does not wait for the disk."""

    def __init__(self):
        super().__init__(daemon=True)
        self.q: queue.Queue = queue.Queue()
        self.errors: list = []
        self.start()

    def run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            fn, args = item
            try:
                fn(*args)
            except Exception as exc:  # reported by close()
                self.errors.append(exc)

    def submit(self, fn, *args):
        self.q.put((fn, args))

    def close(self):
        self.q.put(None)
        self.join()
        if self.errors:
            raise self.errors[0]


class BakeServer:
    def __init__(self, hbm_budget_bytes: int, device: str = "cuda:0", make_solver: Callable | None = None,
                 make_batch: Callable | None = None, clock: Callable[[], float] = time.perf_counter,
                 sort_interval: int | None = None):
        if make_solver is None:
            from mpm_plugin_gb300.solver import Gb300Solver

            def make_solver(job):
                return Gb300Solver(job.domain, job.materials, job.gravity, job.particles_per_cell, device=device)
        if make_batch is None:
            from mpm_plugin_gb300.batch import Gb300Batch

            make_batch = Gb300Batch
        self.budget = int(hbm_budget_bytes)
        self.make_solver = make_solver
        self.batch = make_batch()
        if sort_interval is not None:
            from mpm_plugin_gb300 import _abi

            self.batch.set_option(_abi.OPT_SORT_INTERVAL, sort_interval)
        self.clock = clock
        self.pending: deque = deque()  # (arrival, job), arrival order
        self.runs: list[_Run] = []     # resident jobs, in the batch's scene order
        self.reserved = 0
        self.report = ServeReport()
        self.writer = _Writer()
        self._t0 = clock()

    def now(self) -> float:
        return self.clock() - self._t0

    def submit(self, job: BakeJob, arrival: float | None = None) -> None:
        self.pending.append((self.now() if arrival is None else arrival, job))

    def _admit(self) -> None:
        now = self.now()
        while self.pending and self.pending[0][0] <= now:
            arrival, job = self.pending[0]
            need = estimate_device_bytes(job.domain, job.max_particles, job.collider_triangles)
            if need > self.budget:
                self.pending.popleft()
                self.report.rejected.append(job.name)
                continue
            if self.reserved + need > self.budget:
                # FIFO: wait until resident jobs finish and free their memory
                self.report.max_queue = max(self.report.max_queue, sum(1 for a, _ in self.pending if a <= now))
                return
            self.pending.popleft()
            solver = self.make_solver(job)
            if job.setup:
                job.setup(solver)
            self.batch.add(solver)
            t = self.now()
            self.runs.append(_Run(job, solver, need, arrival, t, last=t))
            self.report.admit_wait_s.append(t - arrival)
            self.reserved += need
        self.report.max_resident = max(self.report.max_resident, len(self.runs))
        self.report.max_reserved = max(self.report.max_reserved, self.reserved)

    def _finish(self, run: _Run, failed: str | None = None) -> None:
        self.batch.remove(run.solver)
        run.solver.close()
        self.runs.remove(run)
        self.reserved -= run.reserved
        if failed:
            self.report.failed[run.job.name] = failed
        else:
            self.report.job_latency_s[run.job.name] = self.now() - run.arrival

    def tick(self) -> bool:
        """Admit what fits, then advance every resident job by one frame. False when nothing is resident."""
        self._admit()
        if not self.runs:
            return False
        t0 = self.clock()
        for run in self.runs:
            if run.job.before_frame:
                run.job.before_frame(run.solver, run.frame + 1)
        counts = [run.solver.particle_count for run in self.runs]
        stats = self.batch.advance([1.0 / run.job.fps for run in self.runs])
        done = []
        # every job's frame read starts at once (each on its own copy stream), then they are collected
        reads = [run.solver.get_particles_async() if hasattr(run.solver, "get_particles_async") else None
                 for run in self.runs]
        for run, n, st, rd in zip(list(self.runs), counts, stats, reads):
            run.frame += 1
            self.report.particle_substeps += n * st.substeps
            if rd is not None:
                a = rd.wait()
                particles = ParticleData(a["x"], a["v"], a["mat"], a["emitter"])
            else:
                particles = run.solver.get_particles()
            if not (np.isfinite(particles.positions).all() and np.isfinite(particles.velocities).all()):
                done.append((run, f"simulation became unstable at frame {run.frame} (NaN/inf in particle positions)"))
                continue
            if run.job.writer is not None:
                self.writer.submit(run.job.writer.write_frame, run.frame, particles)
            t = self.now()
            self.report.frame_latency_ms.append(1e3 * (t - run.last))
            run.last = t
            if run.frame >= run.job.frames:
                done.append((run, None))
        self.report.busy_s += self.clock() - t0
        for run, failed in done:
            self._finish(run, failed)
        return True

    def run(self, trace=(), idle_sleep: float = 1e-3) -> ServeReport:
        """Serve a trace of (arrival seconds from now, job) until every job is done or rejected."""
        for arrival, job in sorted(trace, key=lambda a: a[0]):
            self.submit(job, self.now() + arrival)
        start = self.now()
        while self.pending or self.runs:
            if not self.tick() and self.pending:
                wait = self.pending[0][0] - self.now()
                if wait > 0:
                    time.sleep(min(wait, idle_sleep * 100))
        self.writer.close()
        self.writer = _Writer()
        self.report.wall_s += self.now() - start
        return self.report

    def close(self) -> None:
        for run in list(self.runs):
            self._finish(run, "server closed")
        self.writer.close()
        self.batch.close()

"""Bake server host logic on the CPU, with stand-ins for the solver and the batch: admission against the
device-memory budget, FIFO order, rejection of jobs larger than the budget, frame hand-off order, latency
bookkeeping and the footprint estimate."""

from __future__ import annotations

import numpy as np
from scenes import domain

from mpm_plugin_gb300.interface import AdvanceStats, ParticleData
from mpm_plugin_gb300.serve import BakeJob, BakeServer, estimate_device_bytes


class FakeSolver:
    def __init__(self, job):
        self.job = job
        self.n = 1000
        self.closed = False

    @property
    def particle_count(self):
        return self.n

    def get_particles(self):
        pos = np.zeros((self.n, 3), np.float32)
        return ParticleData(pos, pos.copy(), np.zeros(self.n, np.int32), np.zeros(self.n, np.int32))

    def close(self):
        self.closed = True


class FakeBatch:
    def __init__(self):
        self.scenes = []
        self.max_size = 0
        self.advances = []

    def add(self, s):
        self.scenes.append(s)
        self.max_size = max(self.max_size, len(self.scenes))

    def remove(self, s):
        self.scenes.remove(s)

    def advance(self, frame_dt):
        assert len(frame_dt) == len(self.scenes)
        self.advances.append([s.job.name for s in self.scenes])
        return [AdvanceStats(10, f / 10, 0) for f in frame_dt]

    def close(self):
        pass


class Collect:
    def __init__(self):
        self.frames = []

    def write_frame(self, frame, particles):
        self.frames.append(frame)


def _job(name, frames, res=32, writer=None):
    return BakeJob(name, domain(res=res), [], frames, writer=writer, max_particles=100_000)


def test_footprint_grows_with_particles_and_grid():
    a = estimate_device_bytes(domain(res=32), 100_000)
    assert estimate_device_bytes(domain(res=32), 200_000) > a
    assert estimate_device_bytes(domain(res=64), 100_000) > a
    assert a > 2 * 2 * 100_000 * 136  # two arenas at twice the particle count


def test_admission_respects_budget_and_fifo():
    one = estimate_device_bytes(domain(res=32), 100_000)
    batch = FakeBatch()
    writers = [Collect() for _ in range(4)]
    srv = BakeServer(int(2.5 * one), make_solver=FakeSolver, make_batch=lambda: batch)
    jobs = [_job(f"j{i}", 3 + i, writer=writers[i]) for i in range(4)]
    big = BakeJob("huge", domain(res=32), [], 2, max_particles=10**9)
    rep = srv.run([(0.0, j) for j in jobs] + [(0.0, big)])
    srv.close()
    assert batch.max_size == 2 and rep.max_resident == 2
    assert rep.max_reserved <= srv.budget
    assert rep.rejected == ["huge"]
    assert sorted(rep.job_latency_s) == ["j0", "j1", "j2", "j3"]
    # FIFO: j2 is admitted when j0 (the shortest) finishes, j3 when the next one does
    first = [names for names in batch.advances if "j2" in names][0]
    assert "j0" not in first and "j1" in first
    for i, w in enumerate(writers):
        assert w.frames == list(range(1, 4 + i))  # every frame, in order
    assert len(rep.frame_latency_ms) == sum(3 + i for i in range(4))
    assert rep.particle_substeps == 1000 * 10 * sum(3 + i for i in range(4))


def test_unstable_job_fails_alone():
    class NanSolver(FakeSolver):
        def get_particles(self):
            p = super().get_particles()
            if self.job.name == "bad":
                p.positions[0] = np.nan
            return p

    batch = FakeBatch()
    srv = BakeServer(10**12, make_solver=NanSolver, make_batch=lambda: batch)
    rep = srv.run([(0.0, _job("bad", 5)), (0.0, _job("good", 3))])
    srv.close()
    assert "unstable at frame 1" in rep.failed["bad"]
    assert "good" in rep.job_latency_s

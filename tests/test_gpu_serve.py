"""The bake server on the GPU: every job's frames are the same whether it is baked alone (the bake runner's
loop over one solver) or in the mix with jobs that arrive while it runs, within the float-summation
tolerance; its writer receives every frame in order."""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import add, box_particles, domain, icosphere, lattice_box, preset, rot_x, scale, translate

from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
from mpm_plugin_gb300.serve import BakeJob, BakeServer

pytestmark = pytest.mark.gpu


class Collect:
    def __init__(self):
        self.frames = {}

    def write_frame(self, frame, particles):
        self.frames[frame] = particles.positions.copy()


def _jobs():
    d1, d2, d3 = domain(res=32), domain(res=48), domain(res=40)
    ball = icosphere(1.0, 3)

    def setup_jelly(s):
        add(s, box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d1.dx, seed=1), 0, 0, (0.5, 0.0, 0.0))

    def setup_sand(s):
        add(s, box_particles((0.25, 0.25, 0.0), (0.75, 0.75, 0.12), d2.dx, seed=2))
        s.set_colliders([ColliderGeometry(MeshData(*ball), closed=True, friction=0.2)])

    def spin(s, k):  # a sphere rolling through the sand, per-frame world matrices (start, end)
        xf = [translate(0.3 + 0.02 * f, 0.5, 0.1) @ rot_x(20.0 * f) @ scale(0.1) for f in (k - 1, k)]
        s.set_collider_transforms(xf[0][None], xf[1][None])

    def pour(s, k):  # inflow: a slab above the pile, added where no material is
        rng = np.random.default_rng(100 + k)
        slab = lattice_box((0.45, 0.45, 0.8), (0.55, 0.55, 0.82), d3.dx / 2, rng)
        free = ~s.is_occupied(slab)
        if free.any():
            p = slab[free]
            s.add_particles(p, np.tile(np.float32([0, 0, -2.0]), (len(p), 1)), np.zeros(len(p), np.int32),
                            np.zeros(len(p), np.int32))

    return [BakeJob("jelly", d1, [preset("jelly")], 6, setup=setup_jelly, writer=Collect(), max_particles=40_000),
            BakeJob("sand", d2, [preset("sand_dry")], 5, setup=setup_sand, before_frame=spin, writer=Collect(),
                    max_particles=120_000, collider_triangles=1280),
            BakeJob("pour", d3, [preset("sand_dry")], 6, before_frame=pour, writer=Collect(), max_particles=40_000)]


def _alone(job):
    from mpm_plugin_gb300.solver import Gb300Solver

    s = Gb300Solver(job.domain, job.materials, job.gravity, job.particles_per_cell, device="cuda:0")
    if job.setup:
        job.setup(s)
    for k in range(1, job.frames + 1):
        if job.before_frame:
            job.before_frame(s, k)
        s.advance(1.0 / job.fps)
        job.writer.write_frame(k, s.get_particles())
    s.close()


def test_each_job_same_alone_and_in_the_mix():
    alone, mixed = _jobs(), _jobs()
    for job in alone:
        _alone(job)
    srv = BakeServer(8 << 30)
    srv.submit(mixed[0])
    srv.submit(mixed[1])
    srv.tick()
    srv.tick()
    srv.submit(mixed[2])  # arrives while the others are on the GPU
    rep = srv.run()
    srv.close()
    assert rep.max_resident == 3 and not rep.failed and not rep.rejected
    for a, m in zip(alone, mixed):
        assert sorted(m.writer.frames) == list(range(1, m.frames + 1))
        for k in range(1, m.frames + 1):
            pa, pm = a.writer.frames[k], m.writer.frames[k]
            assert pa.shape == pm.shape, (a.name, k)
            assert rel_err(pm, pa) <= 1e-4, (a.name, k, rel_err(pm, pa))
    assert len(rep.frame_latency_ms) == sum(j.frames for j in mixed)


def test_deterministic_jobs_are_bit_identical_alone_and_in_the_mix():
    """In deterministic mode (fixed-point P2G and occupancy) a job's frames do not depend on what else is in
    the batch: bit-identical to the job baked alone."""
    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.solver import Gb300Solver

    def make(job):
        s = Gb300Solver(job.domain, job.materials, job.gravity, job.particles_per_cell, device="cuda:0")
        s.set_option(_abi.OPT_DETERMINISTIC, 1)
        return s

    alone, mixed = _jobs(), _jobs()
    for job in alone:
        s = make(job)
        if job.setup:
            job.setup(s)
        for k in range(1, job.frames + 1):
            if job.before_frame:
                job.before_frame(s, k)
            s.advance(1.0 / job.fps)
            job.writer.write_frame(k, s.get_particles())
        s.close()
    srv = BakeServer(8 << 30, make_solver=make)
    srv.submit(mixed[0])
    srv.submit(mixed[1])
    srv.tick()
    srv.submit(mixed[2])
    rep = srv.run()
    srv.close()
    assert rep.max_resident == 3 and not rep.failed
    for a, m in zip(alone, mixed):
        for k in range(1, m.frames + 1):
            np.testing.assert_array_equal(m.writer.frames[k], a.writer.frames[k], err_msg=f"{a.name} frame {k}")

"""The reference's unchanged bake runner (mpm_core.bake, bake.py:116-213) end to end on the CPU, with the FP32
oracle registered as an mpm_core backend (test infrastructure; it stands in for a backend here because the
runner is backend-neutral). An inflow scene with a moving collider is baked with the runner's own synchronous
frame and checkpoint writes, and again with install_async_io (the writer thread mpm_plugin_gb300.bake puts
around the runner): the two caches hold the same files with byte-identical contents. Skipped where mpm_core
is not importable."""

from __future__ import annotations

import numpy as np
import pytest
from scenes import bake_scene, cache_contents

runner = pytest.importorskip("mpm_core.bake", reason="the reference package mpm_core is not importable")


def _oracle_backend():
    from mpm_core.solver import AdvanceStats, ParticleData, Solver

    from oracle.oracle import OracleSolver

    class OracleBackend(Solver):
        """mpm_core.solver.Solver over the FP32 oracle (warp/solver.py's host logic restated around C kernels)."""

        def __init__(self, domain, materials, gravity, particles_per_cell=8, device=None):
            super().__init__(domain, materials, gravity, particles_per_cell, device)
            self.o = OracleSolver(domain, materials, gravity, particles_per_cell, threads=1)  # one thread: the same sums every run

        def add_particles(self, positions, velocities, material_ids, emitter_ids):
            self.o.add_particles(positions, velocities, material_ids, emitter_ids)

        def set_colliders(self, colliders):
            self.o.set_colliders([(c.mesh.verts, c.mesh.tris, c.closed, c.friction) for c in colliders])

        def set_collider_transforms(self, start, end):
            self.o.set_collider_transforms(start, end)

        def advance(self, frame_dt):
            return AdvanceStats(*self.o.advance(frame_dt))

        @property
        def particle_count(self):
            return self.o.particle_count

        def get_particles(self):
            s = self.o.save_state()
            return ParticleData(s["x"], s["v"], s["mat"], s["emitter"])

        def is_occupied(self, points):
            return self.o.is_occupied(points)

        def save_state(self):
            return self.o.save_state()

        def load_state(self, state):
            self.o.load_state(state)

    return OracleBackend


@pytest.fixture
def oracle_backend():
    from mpm_core.backends import register_backend

    cls = _oracle_backend()
    register_backend("oracle", lambda **kw: cls(**kw))
    return "oracle"


def _bake(cache, scene, backend, asynchronous, monkeypatch):
    from mpm_core.cache import CacheReader
    from mpm_core.scene import write_scene

    from mpm_plugin_gb300.bake import install_async_io

    write_scene(scene, cache / "scene")
    with monkeypatch.context() as m:  # the runner module's attributes come back after this bake
        for name in ("CacheWriter", "write_checkpoint", "bake"):
            m.setattr(runner, name, getattr(runner, name))
        writer = install_async_io(runner) if asynchronous else None
        result = runner.bake(cache, backend=backend)
        if writer is not None:
            writer.close()
    assert result.status == "done", result.message
    return CacheReader(cache)


def test_async_writes_give_the_same_cache(tmp_path, oracle_backend, monkeypatch):
    scene = bake_scene(resolution=16, frame_end=4)
    sync = _bake(tmp_path / "sync", scene, oracle_backend, False, monkeypatch)
    asyn = _bake(tmp_path / "async", scene, oracle_backend, True, monkeypatch)
    assert sync.available_frames() == asyn.available_frames() == [1, 2, 3, 4]
    counts = [len(sync.read_frame(f)["pour"][0]) for f in range(1, 5)]
    assert counts[0] > 0 and counts[2] > counts[0] and counts[3] == counts[2]  # emitting over frames 1-3
    a, b = cache_contents(tmp_path / "sync"), cache_contents(tmp_path / "async")
    assert sorted(a) == sorted(b) and "state/checkpoint.npz" in a and "frames/frame_0004.npz" in a
    for k in a:
        assert a[k] == b[k], k


def test_resume_from_the_async_checkpoint(tmp_path, oracle_backend, monkeypatch):
    """A bake cancelled after frame 2 (with asynchronous writes) and resumed gives the uninterrupted bake's
    frames: the checkpoint on disk belongs to the last frame file written."""
    from mpm_core.cache import CacheReader
    from mpm_core.scene import write_scene

    from mpm_plugin_gb300.bake import install_async_io

    scene = bake_scene(resolution=16, frame_end=4)
    full = _bake(tmp_path / "full", scene, oracle_backend, True, monkeypatch)
    cache = tmp_path / "cut"
    write_scene(scene, cache / "scene")
    with monkeypatch.context() as m:
        for name in ("CacheWriter", "write_checkpoint", "bake"):
            m.setattr(runner, name, getattr(runner, name))
        writer = install_async_io(runner)
        calls = iter(range(100))
        assert runner.bake(cache, backend=oracle_backend, should_cancel=lambda: next(calls) >= 1).status == "cancelled"
        assert runner.bake(cache, backend=oracle_backend, resume=True).status == "done"
        writer.close()
    cut = CacheReader(cache)
    assert cut.available_frames() == [1, 2, 3, 4]
    for f in (3, 4):
        np.testing.assert_array_equal(cut.read_frame(f)["pour"][0], full.read_frame(f)["pour"][0])

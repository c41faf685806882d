"""Frame I/O around the bake runner on the CPU: the asynchronous writer keeps the runner's write order and
files, surfaces writer errors on the runner's thread, and the bake returns only after every write."""

from __future__ import annotations

import threading
import time
import types

import numpy as np
import pytest

from mpm_plugin_gb300.bake import FrameWriter, install_async_io


def _fake_runner(log, slow=0.0, fail_at=None, frames=5):
    """A stand-in for the runner module: bake() writes `frames` frames, each followed by its checkpoint
    (bake.py:199-201), through the module's CacheWriter and write_checkpoint."""

    class CacheWriter:
        def __init__(self, cache_dir):
            self.cache_dir = cache_dir

        def write_frame(self, frame, particles):
            time.sleep(slow)
            if fail_at == frame:
                raise OSError("disk full")
            log.append(("frame", frame, threading.current_thread().name, float(particles.sum())))

    def write_checkpoint(cache_dir, frame, state, scene_hash):
        time.sleep(slow)
        log.append(("checkpoint", frame, threading.current_thread().name, float(state["x"].sum())))

    mod = types.SimpleNamespace(CacheWriter=CacheWriter, write_checkpoint=write_checkpoint)

    def bake(cache_dir):
        w = mod.CacheWriter(cache_dir)
        for f in range(1, frames + 1):
            x = np.full((4, 3), float(f), np.float32)
            w.write_frame(f, x)
            mod.write_checkpoint(cache_dir, f, {"x": x}, "hash")  # fresh arrays every frame, as the runner's
        return "done"

    mod.bake = bake
    return mod


def test_async_writes_keep_order_and_content_and_finish_before_return():
    sync_log, async_log = [], []
    assert _fake_runner(sync_log).bake("c") == "done"
    runner = _fake_runner(async_log, slow=0.01)
    writer = install_async_io(runner)
    t0 = time.perf_counter()
    assert runner.bake("c") == "done"
    assert time.perf_counter() - t0 >= 10 * 0.01  # returned only after the writes
    assert [e[:2] + e[3:] for e in async_log] == [e[:2] + e[3:] for e in sync_log]
    assert all(e[2] == "mpm-frame-writer" for e in async_log)
    writer.close()


def test_writer_error_reaches_the_runner_thread():
    log = []
    runner = _fake_runner(log, fail_at=2)
    writer = install_async_io(runner)
    with pytest.raises(OSError, match="disk full"):
        runner.bake("c")
    assert ("frame", 3) not in [e[:2] for e in log]  # nothing is written after the failure
    writer.close()


def test_drain_waits_and_close_stops_the_thread():
    w = FrameWriter()
    out = []
    for i in range(20):
        w.submit(out.append, i)
    w.drain()
    assert out == list(range(20))
    w.close()

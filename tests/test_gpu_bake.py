"""The reference's unchanged bake runner driving the gb300 backend on the GPU (python -m mpm_plugin_gb300.bake,
which runs mpm_core.bake.main with --backend gb300). Ports of the reference's runner tests that need a real
backend (tests/test_bake.py:208-214 inflow, :217-222 the command line, :254-271 the command line stopping
when its parent goes away), and the frame I/O claim on the real backend: in deterministic mode a bake with
the writer thread and device-side emitter sampling writes the same cache, byte for byte, as one with the
runner's own synchronous writes and host sampling. Skipped where mpm_core is not importable."""

from __future__ import annotations

import json
import os
import subprocess
import sys
import time
from pathlib import Path

import pytest
from scenes import bake_scene, cache_contents

pytestmark = pytest.mark.gpu
pytest.importorskip("mpm_core.bake", reason="the reference package mpm_core is not importable")

ROOT = Path(__file__).resolve().parent.parent


def _env():
    """The environment of a runner subprocess: this repository and the mpm_core install on its path."""
    paths = [str(ROOT)] + [p for p in sys.path if (Path(p) / "mpm_core").is_dir()]
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join(paths + [env.get("PYTHONPATH", "")])
    return env


def _write(cache, scene):
    from mpm_core.scene import write_scene

    write_scene(scene, Path(cache) / "scene")


def _run(cache, *flags, timeout=600):
    out = subprocess.run([sys.executable, "-m", "mpm_plugin_gb300.bake", str(cache), "--device", "cuda:0", *flags],
                         capture_output=True, text=True, env=_env(), timeout=timeout)
    assert out.returncode == 0, out.stderr[-2000:]
    return out


def test_inflow_emits_while_active(tmp_path):
    """tests/test_bake.py:208-214 on the gb300 backend: an inflow active over frames 1-10 of 20 grows the
    particle count while active and keeps it afterwards."""
    from mpm_core.cache import CacheReader

    _write(tmp_path, bake_scene(resolution=32, frame_end=20, emit_frames=(1, 10), substeps=1))
    _run(tmp_path)
    r = CacheReader(tmp_path)
    counts = [len(r.read_frame(f)["pour"][0]) for f in range(1, 21)]
    assert counts[9] > counts[1] and counts[10:] == [counts[10]] * 10, counts
    assert json.loads((tmp_path / "cache.json").read_text())["backend"] == "gb300"


def test_writer_thread_and_device_sampling_write_the_same_cache(tmp_path):
    """Deterministic mode: the asynchronous writer with device-side sampling (the defaults) against the
    runner's synchronous writes with its own host sampling: byte-identical frames and checkpoint."""
    scene = bake_scene(resolution=32, frame_end=6, emit_frames=(1, 4), substeps=3)
    _write(tmp_path / "a", scene)
    _write(tmp_path / "b", scene)
    _run(tmp_path / "a", "--deterministic")
    _run(tmp_path / "b", "--deterministic", "--sync-io", "--host-sampling")
    a, b = cache_contents(tmp_path / "a"), cache_contents(tmp_path / "b")
    assert sorted(a) == sorted(b) and "frames/frame_0006.npz" in a and "state/checkpoint.npz" in a
    for k in a:
        assert a[k] == b[k], k


def test_cli_stops_when_parent_goes_away(tmp_path):
    """tests/test_bake.py:254-271: with --watch-stdin the runner stops as if cancelled when its stdin closes
    (what the OS does when the launching process exits), exit code 0, status "cancelled"."""
    _write(tmp_path, bake_scene(resolution=32, frame_end=4000, emit_frames=(1, 1), substeps=1))
    proc = subprocess.Popen([sys.executable, "-m", "mpm_plugin_gb300.bake", str(tmp_path), "--watch-stdin"],
                            stdin=subprocess.PIPE, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env=_env())
    try:
        deadline = time.time() + 120
        while time.time() < deadline:
            try:
                if (json.loads((tmp_path / "progress.json").read_text()).get("frame") or 0) >= 2:
                    break
            except (FileNotFoundError, json.JSONDecodeError, PermissionError):
                pass
            time.sleep(0.05)
        proc.stdin.close()
        assert proc.wait(timeout=120) == 0
    finally:
        if proc.poll() is None:
            proc.kill()
    doc = json.loads((tmp_path / "progress.json").read_text())
    assert doc["status"] == "cancelled" and doc["frame"] < 4000

"""Bake runner entry point with the gb300 backend registered.

    python -m mpm_plugin_gb300.bake CACHE_DIR [--device cuda:0] [--resume] [--watch-stdin] [--host-sampling]
                                    [--sync-io] [--deterministic]

Runs the reference's own, unchanged runner (``mpm_core.bake.main``) with ``--backend gb300`` unless another
backend is named; needs the reference package on the path. Around it:

* unless --host-sampling is given, the runner's emitter volume sampling (its ``sample_mesh_volume``, called
  from ``_emit``, bake.py:65) is the device version of mpm_plugin_gb300.emit, which returns the same points
  bit for bit;
* the gb300 solvers the runner creates read each frame's whole state in one copy, shared by the frame's
  get_particles and save_state (bake.py:195-201);
* with --deterministic the gb300 solvers run in deterministic mode (fixed-point P2G: the same cache, bit for
  bit, on every run of the same scene);
* unless --sync-io is given, the frame files and checkpoints (``CacheWriter.write_frame``,
  ``write_checkpoint``, cache.py:131-160) are written by the same functions on one writer thread, in the
  order the runner asks for them, while the next frame simulates. Every file is still written atomically
  (the reference's own atomic_write_npz), a writer error is raised on the runner's thread at the next write
  it asks for, and the bake returns only once every write has finished. A frame is announced in
  progress.json before its file is on disk; resume works from the last checkpoint on disk, which always
  follows its frame file.
"""

from __future__ import annotations

import queue
import sys
import threading


class FrameWriter:
    """One thread running write callbacks in submission order; errors surface on the submitting thread."""

    def __init__(self):
        self._q: queue.Queue = queue.Queue()
        self._errors: list = []
        self._thread = threading.Thread(target=self._run, name="mpm-frame-writer", daemon=True)
        self._thread.start()

    def _run(self):
        while True:
            item = self._q.get()
            try:
                if item is None:
                    return
                if not self._errors:  # after a failure nothing more is written
                    fn, args = item
                    fn(*args)
            except BaseException as exc:  # re-raised by submit / drain
                self._errors.append(exc)
            finally:
                self._q.task_done()

    def _raise(self):
        if self._errors:
            raise self._errors[0]

    def submit(self, fn, *args):
        self._raise()
        self._q.put((fn, args))

    def drain(self):
        """Waits until every submitted write has finished; raises the first writer error."""
        self._q.join()
        self._raise()

    def close(self):
        self._q.put(None)
        self._thread.join()


def install_async_io(runner, writer: FrameWriter | None = None) -> FrameWriter:
    """Routes the runner module's frame and checkpoint writes through a FrameWriter and makes its bake()
    wait for them before it returns (or raises). `runner` is the mpm_core.bake module, or anything with its
    CacheWriter, write_checkpoint and bake attributes."""
    writer = writer or FrameWriter()
    base_writer, base_checkpoint, base_bake = runner.CacheWriter, runner.write_checkpoint, runner.bake

    class AsyncCacheWriter(base_writer):
        def write_frame(self, frame, particles):
            writer.submit(base_writer.write_frame, self, frame, particles)

    def write_checkpoint(cache_dir, frame, state, scene_hash):
        writer.submit(base_checkpoint, cache_dir, frame, state, scene_hash)

    def bake(*args, **kwargs):
        try:
            result = base_bake(*args, **kwargs)
        except BaseException:
            try:
                writer.drain()
            except BaseException:
                pass  # the runner's own error is the one to report
            raise
        writer.drain()
        return result

    runner.CacheWriter = AsyncCacheWriter
    runner.write_checkpoint = write_checkpoint
    runner.bake = bake
    return writer


def _device_index(argv: list[str]) -> int:
    for i, a in enumerate(argv):
        dev = a.split("=", 1)[1] if a.startswith("--device=") else (argv[i + 1] if a == "--device" and i + 1 < len(argv)
                                                                    else None)
        if dev is not None:
            return int(dev.split(":")[1]) if ":" in dev else 0
    return 0


def main(argv: list[str] | None = None) -> int:
    import mpm_plugin_gb300

    if not mpm_plugin_gb300.register():
        print("error: the mpm_core package (the reference bake runner) is not importable", file=sys.stderr)
        return 1
    import mpm_core.bake as runner
    from mpm_core.backends import register_backend

    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.solver import Gb300Solver

    argv = list(sys.argv[1:] if argv is None else argv)
    deterministic = "--deterministic" in argv
    if deterministic:
        argv.remove("--deterministic")

    def factory(**kw):
        solver = Gb300Solver(**kw, frame_reads=True)
        if deterministic:
            solver.set_option(_abi.OPT_DETERMINISTIC, 1)
        return solver

    register_backend(mpm_plugin_gb300.BACKEND_NAME, factory)
    if "--host-sampling" in argv:
        argv.remove("--host-sampling")
    else:
        from mpm_plugin_gb300 import emit

        device = _device_index(argv)
        runner.sample_mesh_volume = lambda v, t, spacing, seed: emit.sample_mesh_volume(v, t, spacing, seed, device)
    if "--sync-io" in argv:
        argv.remove("--sync-io")
    else:
        install_async_io(runner)
    if "--backend" not in argv:
        argv += ["--backend", mpm_plugin_gb300.BACKEND_NAME]
    return runner.main(argv)


if __name__ == "__main__":
    sys.exit(main())

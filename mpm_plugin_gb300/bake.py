"""Bake runner entry point with the gb300 backend registered.

    python -m mpm_plugin_gb300.bake CACHE_DIR [--device cuda:0] [--resume] [--watch-stdin] [--host-sampling]

Runs the reference's own, unchanged runner (``mpm_core.bake.main``) with ``--backend gb300`` unless another
backend is named; needs the reference package on the path. Unless --host-sampling is given, the runner's
emitter volume sampling (its ``sample_mesh_volume``, called from ``_emit``, bake.py:65) is the device
version of mpm_plugin_gb300.emit, which returns the same points bit for bit.
"""

from __future__ import annotations

import sys


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

    argv = list(sys.argv[1:] if argv is None else argv)
    if "--host-sampling" in argv:
        argv.remove("--host-sampling")
    else:
        from mpm_plugin_gb300 import emit

        device = _device_index(argv)
        runner.sample_mesh_volume = lambda v, t, spacing, seed: emit.sample_mesh_volume(v, t, spacing, seed, device)
    if "--backend" not in argv:
        argv += ["--backend", mpm_plugin_gb300.BACKEND_NAME]
    return runner.main(argv)


if __name__ == "__main__":
    sys.exit(main())

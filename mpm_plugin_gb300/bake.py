"""Bake runner entry point with the gb300 backend registered.

    python -m mpm_plugin_gb300.bake CACHE_DIR [--device cuda:0] [--resume] [--watch-stdin]

Runs the reference's own, unchanged runner (``mpm_core.bake.main``) with ``--backend gb300`` unless another
backend is named; needs the reference package on the path.
"""

from __future__ import annotations

import sys


def main(argv: list[str] | None = None) -> int:
    import mpm_plugin_gb300

    if not mpm_plugin_gb300.register():
        print("error: the mpm_core package (the reference bake runner) is not importable", file=sys.stderr)
        return 1
    from mpm_core.bake import main as bake_main

    argv = list(sys.argv[1:] if argv is None else argv)
    if "--backend" not in argv:
        argv += ["--backend", mpm_plugin_gb300.BACKEND_NAME]
    return bake_main(argv)


if __name__ == "__main__":
    sys.exit(main())

"""Build recipe for the C oracle. TEST INFRASTRUCTURE ONLY.

    python oracle/build.py          # writes oracle/_build/liboracle_f32.so and liboracle_f64.so

Plain gcc on one source file: no cmake, no generated code. -ffp-contract=off keeps the operand rounding of
the reference expressions (no fused multiply-adds), so x86-64 and aarch64 builds give the same numbers.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "mpm_oracle.c"
HDR = HERE / "mpm_oracle.h"
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-Wall"]


def lib_path(precision: str) -> Path:
    return BUILD / f"liboracle_{precision}.so"


def build(force: bool = False) -> None:
    BUILD.mkdir(exist_ok=True)
    for precision, extra in (("f32", []), ("f64", ["-DORACLE_DOUBLE"])):
        out = lib_path(precision)
        if not force and out.exists() and out.stat().st_mtime > max(SRC.stat().st_mtime, HDR.stat().st_mtime):
            continue
        tmp = out.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", *FLAGS, *extra, "-o", str(tmp), str(SRC), "-lm"], check=True)
        os.replace(tmp, out)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built in", BUILD)

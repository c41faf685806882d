"""Build recipe of the in-tree CUDA library ``mpm_plugin_gb300/_build/libmpm_gb300.so`` (sm_103a only).

    python -m mpm_plugin_gb300.build [--force]

Three translation units compiled in parallel with nvcc, then linked into one shared library with the CUDA
runtime linked statically. No cmake, no torch extension machinery.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libmpm_gb300.so"
SOURCES = ["mpm_kernels.cu", "mpm_batch_kernels.cu", "mpm_abi.cu", "mpm_noalloc.cu", "mpm_emit.cu", "mpm_surface.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _inputs() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        [HERE.parent / "include" / "mpm_gb300.h", Path(__file__)]


def up_to_date() -> bool:
    return LIB.exists() and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in _inputs())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    procs, objs = [], []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        cmd = [nvcc, *ARCH, *FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out)
        if p.returncode:
            raise RuntimeError(f"nvcc failed ({p.returncode}): {' '.join(cmd)}")
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

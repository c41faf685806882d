"""Host build of the backend's device math for CPU tests (tests/csrc/device_math_host.cpp)."""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "csrc" / "device_math_host.cpp"
DEPS = [SRC, ROOT / "mpm_plugin_gb300" / "csrc" / "mpm_device.cuh", ROOT / "mpm_plugin_gb300" / "csrc" / "mpm_bvh.h",
        ROOT / "mpm_plugin_gb300" / "csrc" / "mpm_types.h"]
OUT = ROOT / "tests" / "_build" / "libdevice_math_host.so"
_lib = None


def _cuda_include() -> str:
    return str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include")


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not OUT.exists() or OUT.stat().st_mtime < max(p.stat().st_mtime for p in DEPS):
        OUT.parent.mkdir(exist_ok=True)
        tmp = OUT.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", _cuda_include(), "-o", str(tmp),
                        str(SRC)], check=True)
        os.replace(tmp, OUT)
    L = C.CDLL(str(OUT))
    P = C.c_void_p
    L.svd_batch.argtypes = [C.c_int, P, P, P, P, P]
    L.svd_batch.restype = C.c_int
    L.stress_batch.argtypes = [C.c_int, C.c_int, P, C.c_float, C.c_float, P]
    L.mesh_build.argtypes = [C.c_int, P, C.c_int, P]
    L.mesh_build.restype = P
    L.mesh_free.argtypes = [P]
    L.mesh_query.argtypes = [P, C.c_int, P, P, P, P]
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def svd(A):
    A = np.ascontiguousarray(np.asarray(A, np.float32).reshape(-1, 3, 3))
    n = len(A)
    U, V = np.zeros((n, 3, 3), np.float32), np.zeros((n, 3, 3), np.float32)
    s, d = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    fp64 = lib().svd_batch(n, _p(A), _p(U), _p(s), _p(d), _p(V))
    return U, s, d, V, fp64


def stress(F, model, mu, lam):
    F = np.ascontiguousarray(np.asarray(F, np.float32).reshape(-1, 3, 3))
    tau = np.zeros_like(F)
    lib().stress_batch(len(F), model, _p(F), mu, lam, _p(tau))
    return tau


class HostMesh:
    def __init__(self, verts, tris):
        self.v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 3))
        self.t = np.ascontiguousarray(np.asarray(tris, np.int32).reshape(-1, 3))
        self.h = lib().mesh_build(len(self.v), _p(self.v), len(self.t), _p(self.t))

    def query(self, pts):
        pts = np.ascontiguousarray(np.asarray(pts, np.float32).reshape(-1, 3))
        n = len(pts)
        cp, sign, face = np.zeros((n, 3), np.float32), np.zeros(n, np.float32), np.zeros(n, np.int32)
        lib().mesh_query(self.h, n, _p(pts), _p(cp), _p(sign), _p(face))
        return cp, sign, face

    def __del__(self):
        try:
            lib().mesh_free(self.h)
        except Exception:
            pass

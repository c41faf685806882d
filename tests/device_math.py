"""Host build of the backend's device math for CPU tests (tests/csrc/device_math_host.cpp)."""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "csrc" / "device_math_host.cpp"
CSRC = ROOT / "mpm_plugin_gb300" / "csrc"
DEPS = [SRC, *(CSRC / f for f in ("mpm_device.cuh", "mpm_bvh.h", "mpm_types.h", "mpm_host.h", "mpm_substep.cuh")),
        ROOT / "include" / "mpm_gb300.h"]
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
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", _cuda_include(),
                        "-o", str(tmp), str(SRC)], check=True)
        os.replace(tmp, OUT)
    L = C.CDLL(str(OUT))
    P = C.c_void_p
    L.svd_batch.argtypes = [C.c_int, P, P, P, P, P]
    L.svd_warm_batch.argtypes = [C.c_int, P, P, P, P, P, P, P]
    L.svd_batch.restype = C.c_int
    L.stress_batch.argtypes = [C.c_int, C.c_int, P, C.c_float, C.c_float, P]
    L.mesh_build.argtypes = [C.c_int, P, C.c_int, P]
    L.mesh_build.restype = P
    L.mesh_free.argtypes = [P]
    L.mesh_query.argtypes = [P, C.c_int, P, P, P, P]
    L.emu_create.argtypes = [P, P, C.c_int, P, C.c_int]
    L.emu_create.restype = P
    L.emu_destroy.argtypes = [P]
    L.emu_set_colliders.argtypes = [P, C.c_int, P]
    L.emu_set_transforms.argtypes = [P, C.c_int, P, P]
    L.emu_grid_dims.argtypes = [P, P]
    L.emu_substep.argtypes = [P, C.c_int64, P, P, P, P, P, P, C.c_int, P, C.c_double, C.c_double, C.c_double]
    L.emu_substep.restype = C.c_uint
    L.emu_read_grid.argtypes = [P, P]
    L.emu_use_sdf.argtypes = [P, C.c_int]
    L.emu_particle_stress.argtypes = [P, C.c_int64, P, P, P, P]
    L.emu_collider_sdf.argtypes = [P, C.c_int, C.c_float, C.c_int, C.c_int, P, P]
    L.emu_sdf_cells.argtypes = [P, C.c_int, P, P, C.c_int64]
    L.emu_sdf_cells.restype = C.c_int64
    L.host_decompose.argtypes = [P, P, P, P]
    L.host_collider_matrix.argtypes = [P, P, C.c_double, C.c_float, P]
    L.host_project.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P]
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


def svd_warm(A, Q):
    """The G2P path of the SVD from the stored bases Q (n, 4; x y z w): U, s, d, V, the new bases, missed."""
    A = np.ascontiguousarray(np.asarray(A, np.float32).reshape(-1, 3, 3))
    Q = np.ascontiguousarray(np.asarray(Q, np.float32).reshape(-1, 4))
    n = len(A)
    U, V = np.zeros((n, 3, 3), np.float32), np.zeros((n, 3, 3), np.float32)
    s, d, Qo = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
    missed = lib().svd_warm_batch(n, _p(A), _p(Q), _p(U), _p(s), _p(d), _p(V), _p(Qo))
    return U, s, d, V, Qo, missed


def stress(F, model, mu, lam):
    F = np.ascontiguousarray(np.asarray(F, np.float32).reshape(-1, 3, 3))
    tau = np.zeros_like(F)
    lib().stress_batch(len(F), model, _p(F), mu, lam, _p(tau))
    return tau


def decompose(m):
    """(t, q, S) of a world matrix by the library's C++ decomposition (float32 matrix in, float64 out)."""
    m = np.ascontiguousarray(np.asarray(m, np.float32).reshape(4, 4))
    t, q, S = np.zeros(3), np.zeros(4), np.zeros(9)
    lib().host_decompose(_p(m), _p(t), _p(q), _p(S))
    return t, q, S.reshape(3, 3)


def collider_matrix(start, end, s, dx=1.0):
    """The 3x4 pose the kernels evaluate at substep fraction s between world matrices start and end."""
    a = np.ascontiguousarray(np.asarray(start, np.float32).reshape(4, 4))
    b = np.ascontiguousarray(np.asarray(end, np.float32).reshape(4, 4))
    out = np.zeros(12, np.float32)
    lib().host_collider_matrix(_p(a), _p(b), dx, s, _p(out))
    return out.reshape(3, 4)


def project(model, d, params):
    """The FP32 return-mapping projection of singular-value deviations d (n, 3), sig = 1 + d: model 2
    Drucker-Prager with params (mu, lam, alpha), 3 snow with (clamp_lo, clamp_hi). Returns (delta, changed,
    marginal)."""
    d = np.ascontiguousarray(np.asarray(d, np.float32).reshape(-1, 3))
    sig = np.ascontiguousarray(np.float32(1) + d)
    p = np.ascontiguousarray(np.asarray(params, np.float32))
    n = len(d)
    delta, changed, marginal = np.zeros((n, 3), np.float32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    lib().host_project(model, n, _p(sig), _p(d), _p(p), _p(delta), _p(changed), _p(marginal))
    return delta, changed.astype(bool), marginal.astype(bool)


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


class SubstepEmulator:
    """The CUDA backend's substep (mpm_substep.cuh) run on the CPU, one item after another."""

    def __init__(self, domain, materials, gravity=(0.0, 0.0, -9.81), ppc=8, use_sdf=True):
        from mpm_plugin_gb300 import _abi

        d = _abi.MpmDomainDesc()
        for a, ax in enumerate("xyz"):
            d.min[a], d.max[a] = domain.min[a], domain.max[a]
            d.wall_lo[a] = int(bool(domain.walls[f"{ax}-"]))
            d.wall_hi[a] = int(bool(domain.walls[f"{ax}+"]))
        d.resolution, d.wall_friction = domain.resolution, domain.wall_friction
        mats = (_abi.MpmMaterialDesc * len(materials))()
        for i, m in enumerate(materials):
            mats[i] = _abi.MpmMaterialDesc(_abi.MODEL_IDS[m.model], m.youngs_modulus, m.poisson_ratio, m.density,
                                           m.yield_stress, m.friction_angle_deg, m.hardening, m.critical_compression,
                                           m.critical_stretch, m.max_hardening)
        g = (C.c_double * 3)(*gravity)
        self._abi = _abi
        self.h = lib().emu_create(C.byref(d), mats, len(materials), g, ppc)
        lib().emu_use_sdf(self.h, int(use_sdf))
        self.state = None

    def set_colliders(self, colliders):
        """colliders: [(verts, tris, closed, friction), ...]"""
        self._keep = []
        descs = (self._abi.MpmColliderDesc * max(1, len(colliders)))()
        for i, (v, t, closed, fr) in enumerate(colliders):
            v = np.ascontiguousarray(np.asarray(v, np.float32).reshape(-1, 3))
            t = np.ascontiguousarray(np.asarray(t, np.int32).reshape(-1, 3))
            self._keep += [v, t]
            descs[i] = self._abi.MpmColliderDesc(len(v), len(t), v.ctypes.data, t.ctypes.data, int(closed), fr)
        lib().emu_set_colliders(self.h, len(colliders), descs)
        self.n_col = len(colliders)
        eye = np.tile(np.eye(4, dtype=np.float32), (self.n_col, 1, 1))
        self.set_collider_transforms(eye, eye)

    def set_collider_transforms(self, start, end):
        self._xf = [np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 4, 4)) for a in (start, end)]
        lib().emu_set_transforms(self.h, self.n_col, _p(self._xf[0]), _p(self._xf[1]))

    def load_state(self, s):
        n = len(s["x"])
        # copies: the substep updates these in place, and the caller's arrays must stay as they were
        self.state = {"x": np.array(np.asarray(s["x"], np.float32).reshape(n, 3).T, order="C"),
                      "v": np.array(np.asarray(s["v"], np.float32).reshape(n, 3).T, order="C"),
                      "C": np.array(np.asarray(s["C"], np.float32).reshape(n, 9).T, order="C"),
                      "F": np.array(np.asarray(s["F"], np.float32).reshape(n, 9).T, order="C"),
                      "Jp": np.array(s["Jp"], np.float32, order="C").reshape(n),
                      "mat": np.array(s["mat"], np.int32, order="C").reshape(n),
                      "emitter": np.asarray(s["emitter"], np.int32).copy(),
                      "tau": np.zeros((6, n), np.float32)}
        self.stress_valid = False

    def save_state(self):
        s = self.state
        n = len(s["Jp"])
        return {"x": s["x"].T.copy(), "v": s["v"].T.copy(), "C": s["C"].T.reshape(n, 3, 3).copy(),
                "F": s["F"].T.reshape(n, 3, 3).copy(), "Jp": s["Jp"].copy(), "mat": s["mat"].copy(),
                "emitter": s["emitter"].copy()}

    def substep(self, dt, s=1.0, frame_dt=1.0):
        st = self.state
        r = lib().emu_substep(self.h, len(st["Jp"]), _p(st["x"]), _p(st["v"]), _p(st["C"]), _p(st["F"]),
                              _p(st["Jp"]), _p(st["tau"]), int(self.stress_valid), _p(st["mat"]), dt, s, frame_dt)
        self.stress_valid = True
        return r

    def stress_of_state(self):
        """(6, n) stress computed from the current F and Jp alone (what a fresh particle would get)."""
        st = self.state
        n = len(st["Jp"])
        tau = np.zeros((6, n), np.float32)
        lib().emu_particle_stress(self.h, n, _p(st["F"]), _p(st["Jp"]), _p(st["mat"]), _p(tau))
        return tau

    def collider_sdf(self, c, s, pts, use_sdf=True):
        """(normal xyz, phi) of collider c at substep fraction s for world points (phi 1e30: far)."""
        pts = np.ascontiguousarray(np.asarray(pts, np.float32).reshape(-1, 3))
        out = np.zeros((len(pts), 4), np.float32)
        lib().emu_collider_sdf(self.h, c, s, int(use_sdf), len(pts), _p(pts), _p(out))
        return out

    def sdf_cells(self, c=0):
        """Collider c's narrow-band voxel grid as built: (lo, voxel edge, contact cutoff, dims, cells (n, 2) of
        (first candidate, count or -1 far / -2 BVH walk)), all in the collider's local units."""
        desc = np.zeros(8, np.float32)
        n = lib().emu_sdf_cells(self.h, c, _p(desc), None, 0)
        cells = np.zeros((n, 2), np.int32)
        lib().emu_sdf_cells(self.h, c, _p(desc), _p(cells), n)
        return desc[:3], float(desc[3]), float(desc[4]), desc[5:8].astype(int), cells

    def read_grid(self):
        dims = np.zeros(3, np.int32)
        lib().emu_grid_dims(self.h, _p(dims))
        out = np.zeros((*dims, 4), np.float32)
        lib().emu_read_grid(self.h, _p(out))
        return out

    def __del__(self):
        try:
            lib().emu_destroy(self.h)
        except Exception:
            pass

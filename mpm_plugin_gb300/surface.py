"""Surfacing of particle frames on the GPU: the drop-in for the reference's mpm_surface/field.py.

``surface_particles(positions, velocities, spacing, settings, device=None, max_bytes=None)`` has the
reference's signature and result (``SurfaceMesh(verts, tris, vel)``: world-space float32 vertices,
outward-wound int32 triangles, float32 vertex velocities) and its host set-up (field.py:104-125): field
cell = spacing / detail, kernel radius h = 2 spacing smoothing, padding h + 2 cells, the memory budget check
at 56 bytes per cell with its ValueError, the rest density of a particle lattice (field.py:92-101). The
splat, normalisation, marching cubes and velocity sampling run in the library (mpm_surface_* in
include/mpm_gb300.h).

    python -m mpm_plugin_gb300.surface CACHE_DIR [--device cuda:0] [--frames 1 2 ...]

runs the reference's own surface runner (mpm_surface.run.surface) with this surface_particles, so the mesh
cache it writes is the reference's format; the reference package must be importable.
"""

from __future__ import annotations

import ctypes as C
import math
import sys
import types
from dataclasses import dataclass
from itertools import product

import numpy as np

from mpm_plugin_gb300 import _abi

BYTES_PER_CELL = 56  # the reference's budget per field cell (field.py:18-20)

try:  # the reference's records when its package is importable
    from mpm_surface.meshcache import SurfaceMesh
    from mpm_surface.settings import SurfaceSettings
except ImportError:  # data-only stand-ins with the same fields (mpm_surface/meshcache.py, settings.py)
    @dataclass
    class SurfaceMesh:
        verts: np.ndarray
        tris: np.ndarray
        vel: np.ndarray

    @dataclass(frozen=True)
    class SurfaceSettings:
        enabled: bool = True
        detail: float = 1.0
        smoothing: float = 2.0
        iso: float = 0.35


def _empty_mesh() -> "SurfaceMesh":
    return SurfaceMesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32), np.zeros((0, 3), np.float32))


def _kernel(q):
    q = np.asarray(q, np.float64)
    t = 1.0 - q
    return np.where(q < 0.5, 1 - 6 * q ** 2 + 6 * q ** 3, np.where(q < 1, 2 * t ** 3, 0.0))


def rest_density(spacing: float, h: float) -> float:
    """Mean kernel sum of a uniform particle lattice over eight sample offsets (field.py:92-101)."""
    n = math.ceil(h / spacing) + 1
    lattice = np.stack(np.meshgrid(*[np.arange(-n, n + 1)] * 3, indexing="ij"), -1).reshape(-1, 3) * spacing
    offsets = np.array(list(product((0, 0.5), repeat=3))) * spacing
    return float(np.mean([_kernel(np.linalg.norm(lattice - o, axis=1) / h).sum() for o in offsets]))


def _device_index(device) -> int:
    s = str(device or "cuda:0")
    if not s.startswith("cuda"):
        raise ValueError(f"the gb300 surfacer runs on CUDA devices only, got device={device!r}")
    return int(s.split(":")[1]) if ":" in s else 0


def _free_bytes(index: int) -> int:
    try:
        import torch

        return int(torch.cuda.mem_get_info(index)[0])
    except Exception:
        return 8 * 1024 ** 3


class Surfacer:
    """One device surfacer (its stream and the buffers of its last build)."""

    def __init__(self, device=None):
        self._lib = _abi.lib()
        self.index = _device_index(device)
        self._s = C.c_void_p()
        status = self._lib.mpm_surface_create(self.index, C.byref(self._s))
        if status != _abi.MPM_OK:
            raise RuntimeError(f"surfacer creation failed on cuda:{self.index} (status {status})")

    def close(self):
        if self._s.value:
            self._lib.mpm_surface_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        if status != _abi.MPM_OK:
            msg = (self._lib.mpm_surface_last_error(self._s) or b"").decode(errors="replace")
            if status == _abi.MPM_ERR_MEMORY:
                raise MemoryError(msg)
            if status == _abi.MPM_ERR_VALUE:
                raise ValueError(msg)
            raise RuntimeError(msg)

    def upload(self, x, v):
        """Copies the particles to the device; returns their per-axis (min, max) as float32 arrays."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(v, np.float32).reshape(-1, 3)
        lo, hi = np.empty(3, np.float32), np.empty(3, np.float32)
        self._check(self._lib.mpm_surface_upload(self._s, len(x), x.ctypes.data_as(C.c_void_p),
                                                 v.ctypes.data_as(C.c_void_p), lo.ctypes.data_as(C.c_void_p),
                                                 hi.ctypes.data_as(C.c_void_p)))
        return lo, hi

    def build(self, origin, dims, cell, h, inv_rest, iso):
        """Runs the device pipeline on the uploaded particles; returns (verts in grid index units, tris, vel)."""
        o = (C.c_float * 3)(*np.asarray(origin, np.float64).astype(np.float32))
        d = (C.c_int32 * 3)(*[int(a) for a in dims])
        nv, nt = C.c_int64(), C.c_int64()
        self._check(self._lib.mpm_surface_build(self._s, o, d, float(cell), float(1.0 / cell), float(h),
                                                float(inv_rest), float(iso), C.byref(nv), C.byref(nt)))
        verts = np.empty((nv.value, 3), np.float32)
        vel = np.empty((nv.value, 3), np.float32)
        tris = np.empty((nt.value, 3), np.int32)
        self._check(self._lib.mpm_surface_read(self._s, verts.ctypes.data_as(C.c_void_p),
                                               tris.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p)))
        self.dims = tuple(int(a) for a in dims)
        return verts, tris, vel

    def read_field(self):
        """(normalised density (dims), field (dims + (4,)): velocity xyz, raw density) of the last build."""
        dens = np.empty(self.dims, np.float32)
        fld = np.empty(self.dims + (4,), np.float32)
        self._check(self._lib.mpm_surface_read_field(self._s, dens.ctypes.data_as(C.c_void_p),
                                                     fld.ctypes.data_as(C.c_void_p)))
        return dens, fld


_surfacers: dict = {}


def _surfacer(device) -> Surfacer:
    i = _device_index(device)
    if i not in _surfacers:
        _surfacers[i] = Surfacer(f"cuda:{i}")
    return _surfacers[i]


def surface_particles(positions: np.ndarray, velocities: np.ndarray, spacing: float, settings,
                      device: str | None = None, max_bytes: int | None = None) -> SurfaceMesh:
    """max_bytes defaults to 70% of the device's currently free memory (field.py:104-142)."""
    positions = np.asarray(positions, np.float32).reshape(-1, 3)
    if len(positions) == 0:
        return _empty_mesh()
    index = _device_index(device)
    surfacer = _surfacer(index)
    # the particles go to the device once; their bounds come back from there (numpy's min and max over
    # axis 0 of an (N, 3) array take longer than the whole surfacing on the GPU)
    lo, hi = surfacer.upload(positions, velocities)
    cell = spacing / settings.detail
    h = 2.0 * spacing * settings.smoothing
    pad = h + 2.0 * cell
    origin = lo.astype(np.float64) - pad
    dims = tuple(int(math.ceil(e / cell)) + 1 for e in hi + pad - origin)
    cells = dims[0] * dims[1] * dims[2]
    needed = cells * BYTES_PER_CELL
    if max_bytes is None:
        max_bytes = int(0.7 * _free_bytes(index))
    if needed > max_bytes:
        raise ValueError(f"surfacing needs a {dims[0]}x{dims[1]}x{dims[2]} grid ({cells:,} cells, about "
                         f"{needed / 1e9:.1f} GB of GPU memory), over the budget of {max_bytes / 1e9:.1f} GB; "
                         f"lower the detail or split the emitter")
    verts, tris, vel = surfacer.build(origin, dims, cell, h, 1.0 / rest_density(spacing, h), settings.iso)
    if len(verts) == 0:
        return _empty_mesh()
    world = (origin + verts.astype(np.float64) * cell).astype(np.float32)
    return SurfaceMesh(world, np.ascontiguousarray(tris), vel)


def install(device: str | None = None) -> None:
    """Makes ``mpm_surface.field`` this module's surface_particles (a stand-in module, so the reference's
    warp-based field module is never imported) before the surface runner is imported."""
    mod = types.ModuleType("mpm_surface.field")
    mod.BYTES_PER_CELL = BYTES_PER_CELL
    mod.surface_particles = lambda p, v, s, st, device_=None, max_bytes=None: surface_particles(
        p, v, s, st, device_ or device, max_bytes)
    sys.modules["mpm_surface.field"] = mod


def main(argv: list[str] | None = None) -> int:
    import argparse
    from pathlib import Path

    ap = argparse.ArgumentParser(prog="python -m mpm_plugin_gb300.surface")
    ap.add_argument("cache_dir", type=Path)
    ap.add_argument("--device", default="cuda:0")
    ap.add_argument("--frames", type=int, nargs="*", default=None)
    args = ap.parse_args(argv)
    install(args.device)
    try:
        from mpm_surface.run import surface
    except ImportError:
        print("error: the mpm_surface package (the reference surface runner) is not importable", file=sys.stderr)
        return 1
    result = surface(args.cache_dir, frames=args.frames, device=args.device)
    print(f"{result.status}: {result.frames_written} frames written, {result.frames_skipped} skipped. "
          f"{result.message}".strip())
    return 1 if result.status == "error" else 0


if __name__ == "__main__":
    sys.exit(main())

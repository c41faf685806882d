"""Emitter volume sampling with the ray-parity test on the GPU (mpm_core/geometry.py:89-155).

sample_mesh_volume(verts, tris, spacing, seed) returns what the reference's function returns, bit for bit:
the same cell-centred lattice, the same inside test (z-ray parity per (x, y) column, the column centre
nudged by the same constant) and the same seeded jitter in the same point order. The reference runs its
per-triangle test in a Python loop on the host; here the triangle-column tests, the crossing sort and the
parity walk run in mpm_volume_lattice, and the host keeps only the lattice set-up, the closedness check and
the jitter (numpy's PCG64 stream, which the points' order must match).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from mpm_plugin_gb300 import _abi

# The reference's ray nudge in units of the spacing (geometry.py:11); the same value is needed for the same
# inside decisions on meshes whose edges lie on lattice columns.
RAY_NUDGE = np.array([1.234567e-4, 2.345678e-4])


def mesh_is_closed(tris) -> bool:
    """True if every undirected edge is shared by exactly two triangles (geometry.py:14-22)."""
    tris = np.asarray(tris)
    if len(tris) == 0:
        return False
    edges = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
    _, counts = np.unique(edges, axis=0, return_counts=True)
    return bool((counts == 2).all())


def sample_mesh_volume(verts, tris, spacing: float, seed, device: int = 0) -> np.ndarray:
    """Points inside a closed mesh on a cell-centred lattice, jittered by +-0.25 spacing (float32, (N, 3))."""
    if not mesh_is_closed(tris):
        raise ValueError("emitter mesh is not closed (every edge must be shared by exactly two triangles)")
    v = np.asarray(verts, np.float64)
    tri = np.ascontiguousarray(v[np.asarray(tris)], np.float64)  # (T, 3, 3)
    lo, hi = v.min(0), v.max(0)
    first = np.ceil(lo / spacing - 0.5).astype(np.int64)
    last = np.floor(hi / spacing - 0.5).astype(np.int64)
    if (last < first).any():
        return np.zeros((0, 3), np.float32)
    xs, ys, zs = [np.ascontiguousarray((np.arange(first[a], last[a] + 1) + 0.5) * spacing) for a in range(3)]
    nudge = np.ascontiguousarray(RAY_NUDGE * spacing, np.float64)
    lib = _abi.lib()
    n = C.c_int64()
    args = [tri.ctypes.data_as(C.c_void_p), len(tri), xs.ctypes.data_as(C.c_void_p), len(xs),
            ys.ctypes.data_as(C.c_void_p), len(ys), zs.ctypes.data_as(C.c_void_p), len(zs), float(spacing),
            nudge.ctypes.data_as(C.c_void_p), int(first[0]), int(first[1]), int(device)]
    _abi.check(lib.mpm_volume_lattice(*args, None, 0, C.byref(n)))
    if n.value == 0:
        return np.zeros((0, 3), np.float32)
    pts = np.empty((n.value, 3), np.float64)
    _abi.check(lib.mpm_volume_lattice(*args, pts.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
    pts += np.random.default_rng(seed).uniform(-0.25, 0.25, pts.shape) * spacing
    return pts.astype(np.float32)

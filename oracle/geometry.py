"""numpy restatement of the reference's host-side geometry on the MPM path. TEST INFRASTRUCTURE ONLY.

Used by the tests (to build seeded scenes without the reference checkout) and by the oracle solver
(collider pose decomposition). Pinned against the reference by ``tests/golden/geometry.npz``.

  mesh_is_closed        mpm_core/geometry.py:14-22
  transform_points      mpm_core/geometry.py:24-27
  decompose_transform   mpm_core/geometry.py:30-50   (polar split M = [R S | t], quaternion x, y, z, w)
  interpolate_transform mpm_core/geometry.py:53-86   (slerp the rotation, lerp stretch and translation)
  sample_mesh_volume    mpm_core/geometry.py:89-155  (z-ray parity on a cell-centred lattice, seeded jitter)
  emission_times        mpm_core/bake.py:100-113
"""

from __future__ import annotations

from fractions import Fraction

import numpy as np

# Lattice rays are moved off the exact column by these fractions of the spacing so that they do not run
# through mesh edges or vertices; the same constants as the reference, so the same points come out.
RAY_NUDGE = np.array([1.234567e-4, 2.345678e-4])


def mesh_is_closed(tris) -> bool:
    tris = np.asarray(tris)
    if len(tris) == 0:
        return False
    e = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    return bool(np.all(counts == 2))


def transform_points(matrix, points) -> np.ndarray:
    m = np.asarray(matrix, np.float64)
    return (np.asarray(points, np.float64) @ m[:3, :3].T + m[:3, 3]).astype(np.float32)


def quat_from_rotation(R) -> np.ndarray:
    """Unit quaternion (x, y, z, w) of a proper rotation: magnitudes from the diagonal, signs from the skew part."""
    tr = (R[0, 0], R[1, 1], R[2, 2])
    w = np.sqrt(max(0.0, 1 + tr[0] + tr[1] + tr[2])) / 2
    x = np.copysign(np.sqrt(max(0.0, 1 + tr[0] - tr[1] - tr[2])) / 2, R[2, 1] - R[1, 2])
    y = np.copysign(np.sqrt(max(0.0, 1 - tr[0] + tr[1] - tr[2])) / 2, R[0, 2] - R[2, 0])
    z = np.copysign(np.sqrt(max(0.0, 1 - tr[0] - tr[1] + tr[2])) / 2, R[1, 0] - R[0, 1])
    q = np.array([x, y, z, w])
    return q / np.linalg.norm(q)


def rotation_from_quat(q) -> np.ndarray:
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def decompose_transform(m):
    """(translation, rotation quaternion, symmetric stretch); a mirror goes into the stretch, not R."""
    A = np.asarray(m, np.float64)[:3, :3]
    U, sig, Vt = np.linalg.svd(A)
    if np.linalg.det(U @ Vt) < 0:
        U[:, 2] *= -1
        sig[2] *= -1
    R = U @ Vt
    S = Vt.T @ np.diag(sig) @ Vt
    return np.asarray(m, np.float64)[:3, 3].copy(), quat_from_rotation(R), S


def slerp(q0, q1, s: float) -> np.ndarray:
    if np.dot(q0, q1) < 0:
        q1 = -q1
    ang = np.arccos(min(float(np.dot(q0, q1)), 1.0))
    if ang < 1e-6:
        q = q0 + s * (q1 - q0)
    else:
        q = (np.sin((1 - s) * ang) * q0 + np.sin(s * ang) * q1) / np.sin(ang)
    return q / np.linalg.norm(q)


def interpolate_transform(a, b, s: float) -> np.ndarray:
    if s == 0:
        return np.asarray(a, np.float32)
    if s == 1:
        return np.asarray(b, np.float32)
    t0, q0, S0 = decompose_transform(a)
    t1, q1, S1 = decompose_transform(b)
    m = np.eye(4)
    m[:3, :3] = rotation_from_quat(slerp(q0, q1, s)) @ (S0 + s * (S1 - S0))
    m[:3, 3] = t0 + s * (t1 - t0)
    return m.astype(np.float32)


def sample_mesh_volume(verts, tris, spacing: float, seed) -> np.ndarray:
    """Lattice points (i + 0.5) * spacing inside a closed mesh, then jittered by U(-0.25, 0.25) * spacing.

    For every lattice column (x, y) the z-crossings of the nudged vertical ray with the mesh are collected;
    a lattice z is inside when an odd number of crossings lie below it. Points come out column by column
    (x index major, y minor), z ascending, and the jitter is drawn for all of them at once.
    """
    if not mesh_is_closed(tris):
        raise ValueError("emitter mesh is not closed (every edge must be shared by exactly two triangles)")
    v = np.asarray(verts, np.float64)
    tri = v[np.asarray(tris)]
    lo_idx = np.ceil(v.min(0) / spacing - 0.5).astype(np.int64)
    hi_idx = np.floor(v.max(0) / spacing - 0.5).astype(np.int64)
    if np.any(hi_idx < lo_idx):
        return np.zeros((0, 3), np.float32)
    axes = [(np.arange(lo_idx[a], hi_idx[a] + 1) + 0.5) * spacing for a in range(3)]
    xs, ys, zs = axes
    ny = len(ys)
    nudge = RAY_NUDGE * spacing

    cols_all, z_all = [], []
    for a, b, c in tri:
        bb_lo = np.minimum(np.minimum(a, b), c)[:2]
        bb_hi = np.maximum(np.maximum(a, b), c)[:2]
        i0 = max(int(np.ceil((bb_lo[0] - nudge[0]) / spacing - 0.5)) - lo_idx[0], 0)
        i1 = min(int(np.floor((bb_hi[0] - nudge[0]) / spacing - 0.5)) - lo_idx[0], len(xs) - 1)
        j0 = max(int(np.ceil((bb_lo[1] - nudge[1]) / spacing - 0.5)) - lo_idx[1], 0)
        j1 = min(int(np.floor((bb_hi[1] - nudge[1]) / spacing - 0.5)) - lo_idx[1], ny - 1)
        if i1 < i0 or j1 < j0:
            continue
        area = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])
        if area == 0.0:
            continue  # a vertical triangle is never crossed by a vertical ray
        ii, jj = np.meshgrid(np.arange(i0, i1 + 1), np.arange(j0, j1 + 1), indexing="ij")
        px, py = xs[ii] + nudge[0], ys[jj] + nudge[1]
        w0 = ((b[0] - px) * (c[1] - py) - (b[1] - py) * (c[0] - px)) / area
        w1 = ((c[0] - px) * (a[1] - py) - (c[1] - py) * (a[0] - px)) / area
        w2 = 1.0 - w0 - w1
        hit = (w0 >= 0) & (w1 >= 0) & (w2 >= 0)
        if hit.any():
            cols_all.append((ii[hit] * ny + jj[hit]).ravel())
            z_all.append((w0 * a[2] + w1 * b[2] + w2 * c[2])[hit].ravel())
    if not cols_all:
        return np.zeros((0, 3), np.float32)
    cols = np.concatenate(cols_all)
    z = np.concatenate(z_all)
    order = np.lexsort((z, cols))
    cols, z = cols[order], z[order]
    bounds = np.flatnonzero(np.diff(cols)) + 1
    pieces = []
    for seg_cols, seg_z in zip(np.split(cols, bounds), np.split(z, bounds)):
        below = np.searchsorted(seg_z, zs)
        zin = zs[below % 2 == 1]
        if len(zin):
            col = seg_cols[0]
            pieces.append(np.column_stack([np.full(len(zin), xs[col // ny]), np.full(len(zin), ys[col % ny]), zin]))
    if not pieces:
        return np.zeros((0, 3), np.float32)
    pts = np.concatenate(pieces)
    pts += np.random.default_rng(seed).uniform(-0.25, 0.25, pts.shape) * spacing
    return pts.astype(np.float32)


def emission_times(emitters, frame: int):
    """[(Fraction of the frame, [emitter index, ...]), ...] in time order, always ending at 1.

    ``emitters``: sequence of (kind, frame_start, frame_end, substeps).
    """
    times: dict[Fraction, list[int]] = {Fraction(1): []}
    for i, (kind, f0, f1, sub) in enumerate(emitters):
        if kind != "inflow" or not f0 <= frame <= f1:
            continue
        for j in (range(1, sub + 1) if frame > f0 else [sub]):
            times.setdefault(Fraction(j, sub), []).append(i)
    return sorted(times.items())

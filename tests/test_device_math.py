"""The backend's device math built for the host (CPU only): SVD accuracy, stress accuracy, mesh queries, and
the collider pose decomposition and interpolation against the reference's recorded outputs."""

from __future__ import annotations

import json

import numpy as np
import pytest
from _golden import GOLDEN
from device_math import HostMesh, stress, svd
from scenes import icosphere, plane_mesh, unit_cube_mesh

from oracle.oracle import OracleMesh


def _rand_F(n, scale, seed):
    rng = np.random.default_rng(seed)
    return (np.eye(3) + scale * rng.normal(size=(n, 3, 3))).astype(np.float32)


@pytest.mark.parametrize("scale", [1e-4, 1e-2, 0.3])
def test_svd_convention_and_accuracy(scale):
    F = _rand_F(20000, scale, 1)
    U, s, d, V, fp64 = svd(F)
    F64 = F.astype(np.float64)
    rec = np.einsum("nij,nj,nkj->nik", U.astype(np.float64), s.astype(np.float64), V.astype(np.float64))
    # reconstruction within 4e-6 of each matrix's largest entry (about 30 FP32 ulps)
    size = np.maximum(np.abs(F64).max(axis=(1, 2)), 1.0)
    assert (np.abs(rec - F64).max(axis=(1, 2)) / size).max() < 4e-6
    assert np.allclose(np.linalg.det(U), 1, atol=1e-5) and np.allclose(np.linalg.det(V), 1, atol=1e-5)
    assert (s[:, 0] >= s[:, 1] - 1e-6).all() and (s[:, 1] >= np.abs(s[:, 2]) - 1e-6).all()
    assert (np.sign(s[:, 2]) == np.sign(np.linalg.det(F64))).all()
    # d = sigma - 1 keeps its relative accuracy for small strains
    s_exact = np.linalg.svd(F64, compute_uv=False)
    s_exact[:, 2] *= np.sign(np.linalg.det(F64))
    err = np.abs(d.astype(np.float64) - (s_exact - 1.0))
    assert (err <= 1e-6 * np.abs(s_exact - 1.0) + 1e-7 * scale).mean() > 0.99
    assert fp64 <= 0.01 * len(F)


def test_svd_inverted_and_degenerate():
    F = np.array([np.eye(3), np.diag([1.1, 0.95, -0.9]), np.diag([1.2, 1.2, 0.9]), np.diag([1e-6, 1.0, 1.0]),
                  [[0, 1, 0], [1, 0, 0], [0, 0, 1]], np.zeros((3, 3))], np.float32)
    U, s, d, V, _ = svd(F)
    rec = np.einsum("nij,nj,nkj->nik", U, s, V)
    assert np.abs(rec - F).max() < 1e-5
    assert s[1, 2] < 0 and s[4, 2] < 0  # det < 0: the last singular value carries the sign


@pytest.mark.parametrize("model", [0, 1])
def test_stress_small_strain_accuracy(model):
    """Kirchhoff stress at strains of 1e-4 agrees with the float64 formula to 1e-5 relative."""
    F = _rand_F(5000, 1e-4, 2)
    mu, lam = 2e4, 3e4
    tau = stress(F, model, mu, lam).astype(np.float64)
    F64 = F.astype(np.float64)
    U, s, Vt = np.linalg.svd(F64)
    flip = np.linalg.det(U @ Vt) < 0
    U[flip, :, 2] *= -1
    s[flip, 2] *= -1
    if model == 0:
        R = U @ Vt
        J = np.prod(s, axis=1)
        ref = 2 * mu * (F64 - R) @ np.transpose(F64, (0, 2, 1)) + (lam * J * (J - 1))[:, None, None] * np.eye(3)
    else:
        e = np.log(np.maximum(s, 1e-4))
        g = 2 * mu * e + lam * e.sum(1, keepdims=True)
        ref = np.einsum("nij,nj,nkj->nik", U, g, U)
    rel = np.linalg.norm(tau - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))
    assert np.median(rel) < 1e-5 and rel.max() < 1e-3


@pytest.mark.parametrize("mesh", ["sphere", "cube", "plane"])
def test_mesh_query_matches_oracle(mesh):
    if mesh == "sphere":
        v, t = icosphere(1.0, 2)
    elif mesh == "cube":
        v, t = unit_cube_mesh(centered=True)
    else:
        v, t = plane_mesh(0.8)
    hm, om = HostMesh(v, t), OracleMesh(v, t)
    rng = np.random.default_rng(3)
    pts = [rng.normal(size=(4000, 3)) * 0.7]
    pts.append(np.concatenate([v * r for r in (0.3, 0.9, 1.02)]) + rng.normal(0, 1e-6, (3 * len(v), 3)))
    pts = np.concatenate(pts).astype(np.float32)
    cp, sg, fc = hm.query(pts)
    vv, tt = np.asarray(v, np.float64), np.asarray(t)
    for i, p in enumerate(pts):
        f, s, u, w, d2 = om.query(p.astype(np.float64))
        a, b, c = vv[tt[f]]
        ocp = u * a + w * b + (1 - u - w) * c
        assert sg[i] == s, (i, p)
        assert abs(np.linalg.norm(cp[i].astype(np.float64) - p) - np.sqrt(d2)) < 1e-5
        # the same face, or another face through the same closest point (a shared edge or vertex)
        assert fc[i] == f or np.linalg.norm(cp[i] - ocp) < 1e-5, (i, p, fc[i], f)


@pytest.mark.parametrize("mesh,closed", [("sphere", True), ("cube", True), ("plane", False)])
def test_narrow_band_grid_matches_full_query(mesh, closed):
    """Collider SDF through the narrow-band voxel grid against the full BVH query.

    Where the grid answers "far", the exact distance must be outside and beyond the contact band (or behind
    an open mesh beyond its thickness), so neither grid contact nor particle projection would act; elsewhere
    the two answers are identical.
    """
    from device_math import SubstepEmulator
    from scenes import domain, preset, rot_x, scale, translate

    if mesh == "sphere":
        v, t = icosphere(1.0, 3)
        xf0 = translate(0.5, 0.5, 0.3) @ scale(0.15)
        xf1 = translate(0.5, 0.52, 0.3) @ rot_x(30) @ scale(0.15)
    elif mesh == "cube":
        v, t = unit_cube_mesh(centered=True)
        xf0 = translate(0.5, 0.5, 0.2) @ scale(0.4, 0.3, 0.2)
        xf1 = translate(0.51, 0.5, 0.2) @ rot_x(5) @ scale(0.4, 0.3, 0.2)
    else:
        v, t = plane_mesh(0.8)
        xf0 = translate(0.5, 0.5, 0.3) @ rot_x(10)
        xf1 = xf0
    d = domain(res=64)
    e = SubstepEmulator(d, [preset("jelly")])
    e.set_colliders([(v, t, closed, 0.5)])
    e.set_collider_transforms(xf0[None], xf1[None])
    rng = np.random.default_rng(7)
    pts = rng.uniform(0.0, 1.0, (20000, 3)).astype(np.float32)
    for s in (0.0, 0.5, 1.0):
        a = e.collider_sdf(0, s, pts, use_sdf=True)
        b = e.collider_sdf(0, s, pts, use_sdf=False)
        far = a[:, 3] >= 1e29
        band, thick = d.dx, 2 * d.dx
        # far in the grid: the exact answer is far too, or outside beyond the band
        ok_far = (b[far, 3] >= 1e29) | (b[far, 3] >= band)
        assert ok_far.all()
        np.testing.assert_array_equal(a[~far], b[~far])
        assert (~far).sum() > 100


def test_narrow_band_voxels_list_the_contact_band():
    """The mixed workload's collider (5,120-triangle perturbed sphere, radius 0.12 at 128^3): voxels half the
    contact cutoff wide, at most about 193 per axis, and every voxel within three grid cells of the surface,
    inside or out, answers from a candidate list of at most 128 triangles or as FAR: none falls back to the
    BVH walk, whose one-lane chain was the slowest contact query."""
    from device_math import SubstepEmulator

    from mpm_plugin_gb300.workloads import mixed_scene

    d, mats, _, (cv, ct, xf) = mixed_scene(128, sample=lambda v, t, spacing, seed: np.zeros((1, 3), np.float32))
    e = SubstepEmulator(d, mats)
    e.set_colliders([(cv, ct, True, 0.5)])
    xf = np.asarray(xf, np.float32)
    e.set_collider_transforms(xf[None], xf[None])
    lo, h, cutoff, dims, cells = e.sdf_cells(0)
    assert h == pytest.approx(0.5 * cutoff, rel=1e-6) and dims.max() <= 194
    cell = (1.0 / 128) / 0.12  # one grid cell in the collider's local units
    assert cutoff == pytest.approx(1.25 * cell, rel=1e-4)
    i, j, k = np.meshgrid(*(np.arange(n) for n in dims), indexing="ij")
    centre = np.stack([lo[0] + (i + 0.5) * h, lo[1] + (j + 0.5) * h, lo[2] + (k + 0.5) * h], -1).reshape(-1, 3)
    # the perturbed surface lies within 0.97-1.03 of the centre (vertex jitter 0.03)
    r = np.linalg.norm(centre, axis=1)
    band = (r > 1.03 - 3 * cell) & (r < 0.97 + 3 * cell)
    count = cells[band, 1]
    assert band.sum() > 10000
    assert (count != -2).all() and count.max() <= 128
    listed = count[count > 0]
    assert len(listed) > 0.5 * band.sum() and np.median(listed) < 40


def _closest_point_independent(p, a, b, c):
    """Closest point on a triangle without region tests: the plane projection if it falls inside, else the
    nearest of the closest points on the three edges."""
    n = np.cross(b - a, c - a)
    n2 = n @ n
    q = p - ((p - a) @ n) / n2 * n
    u = np.cross(c - b, q - b) @ n / n2
    v = np.cross(a - c, q - c) @ n / n2
    w = 1 - u - v
    if u >= 0 and v >= 0 and w >= 0:
        return q
    best = None
    for s, e in ((a, b), (b, c), (c, a)):
        t = np.clip((p - s) @ (e - s) / ((e - s) @ (e - s)), 0.0, 1.0)
        x = s + t * (e - s)
        if best is None or (x - p) @ (x - p) < (best - p) @ (best - p):
            best = x
    return best


@pytest.mark.parametrize("mesh", ["sphere", "cube", "plane"])
def test_closest_point_against_independent_method(mesh):
    """Distances of the device query and of the oracle against a closest-point routine with no region logic."""
    v, t = {"sphere": lambda: icosphere(1.0, 1), "cube": lambda: unit_cube_mesh(centered=True),
            "plane": lambda: plane_mesh(0.8)}[mesh]()
    hm, om = HostMesh(v, t), OracleMesh(v, t)
    rng = np.random.default_rng(11)
    pts = (rng.normal(size=(3000, 3)) * 0.8).astype(np.float32)
    tri = np.asarray(v, np.float64)[np.asarray(t)]
    cp, _, _ = hm.query(pts)
    for i, p in enumerate(pts.astype(np.float64)):
        exact = min(np.linalg.norm(_closest_point_independent(p, *tr) - p) for tr in tri)
        assert abs(np.linalg.norm(cp[i] - p) - exact) < 2e-6 * (1 + exact), i
        _, _, _, _, d2 = om.query(p)
        assert abs(np.sqrt(d2) - exact) < 1e-9 * (1 + exact), i


def test_pose_decomposition_matches_reference():
    """The library's C++ decomposition of a collider's world matrix (mpm_host.h decompose, the host side of
    warp/solver.py:154-172) against the reference's geometry.decompose_transform (geometry.py:30-39) on its
    recorded outputs: 24 seeded matrices with non-uniform, uniform and mirrored scales. The quaternion is
    compared up to sign (q and -q are one rotation; the solver flips the end pose to the short way round)."""
    from device_math import decompose

    z = np.load(GOLDEN / "geometry.npz")
    for m, t_ref, q_ref, S_ref in zip(z["mats"], z["t"], z["q"], z["S"]):
        t, q, S = decompose(m)
        np.testing.assert_allclose(t, t_ref, rtol=0, atol=1e-12)
        sign = 1.0 if np.dot(q, q_ref) >= 0 else -1.0
        np.testing.assert_allclose(sign * q, q_ref, rtol=0, atol=1e-12)
        np.testing.assert_allclose(S, S_ref, rtol=0, atol=1e-12 * np.abs(S_ref).max())


def test_collider_pose_matches_reference_interpolation():
    """The pose the kernels evaluate at a substep fraction s (decomposed poses, slerped rotation, lerped
    stretch and translation; colliders.py:30-37) against the reference's geometry.interpolate_transform
    (geometry.py:69-86) on its recorded outputs for 12 matrix pairs at s = 0, 0.25, 0.5, 0.8, 1: the same
    motion up to FP32 rounding."""
    from device_math import collider_matrix

    z = np.load(GOLDEN / "geometry.npz")
    svals = json.loads(str(z["meta"]))["svals"]
    mats = z["mats"]
    for i, row in enumerate(z["interp"]):
        a, b = mats[2 * i], mats[2 * i + 1]
        for s, ref in zip(svals, row):
            M = collider_matrix(a, b, s)
            scale = np.abs(ref[:3]).max()
            np.testing.assert_allclose(M, ref[:3], rtol=0, atol=1e-6 * scale, err_msg=f"pair {i} s {s}")


def test_return_mapping_marginal_decisions():
    """The FP32 projections report as marginal only the decisions whose two outcomes differ by more than
    rounding: the Drucker-Prager separation test near tr eps = 0 with a strain above the floor. The cone, the
    snow clamps and nearly equal log singular values are continuous and never marginal; an undeformed particle
    has no decision to make, nor one whose strains are a few ulps that cancel in tr."""
    from device_math import project

    mu, lam, alpha = 4.0e5, 6.0e5, 0.3
    e_tr0 = -2.0 * np.log1p(1e-3) - 1e-9  # tr eps about -1e-9 against |eps| of 4e-3
    d = np.array([[0.0, 0.0, 0.0],  # undeformed
                  [1e-3, 1e-3, np.expm1(e_tr0)],  # at the separation test
                  [-0.05, 0.02, 0.01],  # compressed and sheared: projected onto the cone
                  [-0.05 * (1 + 1e-7), -0.05, -0.05 * (1 - 1e-7)],  # hydrostatic: no deviatoric direction
                  [0.01, 0.02, 0.005],  # stretched: separation
                  [2 ** -23, -(2 ** -23), 0.0]])  # strains of an ulp, cancelling in tr
    delta, changed, marginal = project(2, d, (mu, lam, alpha))
    assert marginal.tolist() == [False, True, False, False, False, False]
    assert changed[2] and changed[4] and not changed[3]
    np.testing.assert_array_equal(delta[4], -np.float32(d[4]))
    # the cone projection continuous in d: a rounding-sized change of d moves delta by about as much
    d2 = d[2:3] * np.float32(1 + 2 ** -22)
    np.testing.assert_allclose(project(2, d2, (mu, lam, alpha))[0], delta[2:3], rtol=0, atol=1e-7)

    lo, hi = 1 - 0.025, 1 + 0.0045
    ds = np.array([[0.0, 0.0, 0.0], [0.0045, 0.0, 0.0], [-0.025, 0.001, 0.0], [0.01, -0.03, 0.002]])
    delta, changed, marginal = project(3, ds, (lo, hi))
    assert not marginal.any()
    assert changed.tolist() == [False, False, False, True]


def test_svd_from_the_stored_basis():
    """The G2P path of the SVD: started from the previous substep's right basis (a unit quaternion), from the
    identity, or from a garbage quaternion (a cold start), it gives the cold SVD's singular values and a
    reconstruction of F within the same bounds, and returns its basis as a quaternion that rebuilds V."""
    from device_math import svd_warm

    F = _rand_F(5000, 1e-2, 7)
    _, s0, _, _, _ = svd(F)
    # the previous basis: V of F a step earlier (F perturbed back by a small velocity gradient)
    rng = np.random.default_rng(8)
    C = rng.normal(0.0, 1e-3, (len(F), 3, 3)).astype(np.float32)
    F_prev = np.einsum("nij,njk->nik", np.eye(3, dtype=np.float32) - C, F)
    Q_prev = svd_warm(F_prev, np.tile([0, 0, 0, 1], (len(F), 1)))[4]
    F64 = F.astype(np.float64)
    size = np.maximum(np.abs(F64).max(axis=(1, 2)), 1.0)
    for Q in (Q_prev, np.tile([0, 0, 0, 1], (len(F), 1)), np.full((len(F), 4), np.nan)):
        U, s, d, V, Qo, missed = svd_warm(F, Q)
        rec = np.einsum("nij,nj,nkj->nik", U.astype(np.float64), s.astype(np.float64), V.astype(np.float64))
        assert (np.abs(rec - F64).max(axis=(1, 2)) / size).max() < 4e-6
        np.testing.assert_allclose(s, s0, rtol=0, atol=2e-6)
        assert missed == 0
        # the returned quaternion rebuilds V (unit length, the same rotation)
        assert np.abs(np.linalg.norm(Qo, axis=1) - 1.0).max() < 1e-5
        x, y, z, w = Qo.T.astype(np.float64) / np.linalg.norm(Qo, axis=1)
        R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                      np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                      np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)
        assert np.abs(R - V).max() < 2e-6

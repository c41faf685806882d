"""The GPU surfacer (mpm_surface_* through mpm_plugin_gb300.surface) against the CPU restatement of the
reference's field.py: the splat and normalisation field for field, the mesh vertex for vertex and triangle
for triangle (same case table and order), vertex velocities; the mesh closed and wound outward."""

from __future__ import annotations

import collections

import numpy as np
import pytest

from oracle import surface as S

pytestmark = pytest.mark.gpu


def _blob(n_side=14, spacing=0.01, seed=0):
    rng = np.random.default_rng(seed)
    g = (np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * spacing
    c = g.mean(0)
    pts = g[np.linalg.norm(g - c, axis=1) < 0.45 * n_side * spacing]
    pts = pts + rng.uniform(-0.25, 0.25, pts.shape) * spacing + np.array([0.3, 0.5, 0.2])
    w = np.array([0.0, 0.0, 2.0])
    vel = np.cross(w, pts - pts.mean(0)) + rng.normal(0, 0.05, pts.shape)
    return pts.astype(np.float32), vel.astype(np.float32), spacing


def _manifold_errors(tris):
    cnt = collections.Counter()
    for a, b, c in tris:
        for e in ((a, b), (b, c), (c, a)):
            cnt[e] += 1
    return sum(1 for (a, b), n in cnt.items() if n != 1 or cnt.get((b, a), 0) != 1)


@pytest.mark.parametrize("detail,smoothing,iso", [(1.0, 2.0, 0.35), (1.5, 1.5, 0.5)])
def test_surface_matches_oracle(detail, smoothing, iso):
    from mpm_plugin_gb300.surface import SurfaceSettings, _surfacer, surface_particles

    pts, vel, spacing = _blob()
    mesh = surface_particles(pts, vel, spacing, SurfaceSettings(detail=detail, smoothing=smoothing, iso=iso),
                             device="cuda:0")
    dens, fld = _surfacer("cuda:0").read_field()
    ref = S.surface_particles(pts, vel, spacing, detail, smoothing, iso)
    assert dens.shape == tuple(ref["dims"])
    scale = float(ref["density"].max())
    assert np.abs(dens - ref["density"]).max() <= 1e-5 * scale
    raw = fld[..., 3]
    mask = raw > 1e-3 * raw.max()
    dv = fld[..., :3][mask] - ref["velocity"][mask]
    assert np.linalg.norm(dv) <= 1e-5 * np.linalg.norm(ref["velocity"][mask])
    assert len(mesh.verts) == len(ref["verts"]) > 100
    np.testing.assert_array_equal(mesh.tris, ref["tris"])
    assert np.abs(mesh.verts - ref["verts"]).max() <= 1e-4 * ref["cell"]
    assert np.linalg.norm(mesh.vel - ref["vel"]) <= 1e-4 * np.linalg.norm(ref["vel"])
    assert mesh.verts.dtype == np.float32 and mesh.tris.dtype == np.int32 and mesh.vel.dtype == np.float32
    assert _manifold_errors(mesh.tris) == 0
    v = mesh.verts.astype(np.float64)[mesh.tris]
    volume = np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])).sum() / 6.0
    assert volume > 0  # wound outward


def test_budget_error_and_bounds_match_numpy():
    from mpm_plugin_gb300.surface import SurfaceSettings, _surfacer, surface_particles

    pts = np.random.default_rng(0).normal(0, 1, (100_000, 3)).astype(np.float32)
    lo, hi = _surfacer("cuda:0").upload(pts, pts)
    np.testing.assert_array_equal(lo, pts.min(0))
    np.testing.assert_array_equal(hi, pts.max(0))
    pts[7, 1] = np.nan
    lo, hi = _surfacer("cuda:0").upload(pts, pts)
    assert np.isnan(lo[1]) and np.isnan(hi[1]) and not np.isnan(lo[0])
    with pytest.raises(ValueError, match="surfacing needs a"):
        surface_particles(pts[10:110] * 0.01, pts[10:110], 0.0001, SurfaceSettings(), device="cuda:0",
                          max_bytes=1 << 20)


def test_large_blob_is_closed():
    from mpm_plugin_gb300.surface import SurfaceSettings, surface_particles

    rng = np.random.default_rng(3)
    pts = rng.normal(0, 0.05, (200_000, 3)).astype(np.float32) + 0.5
    vel = rng.normal(0, 1, pts.shape).astype(np.float32)
    mesh = surface_particles(pts, vel, 0.004, SurfaceSettings(), device="cuda:0")
    assert len(mesh.tris) > 1000 and _manifold_errors(mesh.tris) == 0
    assert np.isfinite(mesh.verts).all() and np.isfinite(mesh.vel).all()

"""The surfacer's field stage pinned to the reference: mpm_surface/field.py's own surface_particles, its splat,
normalize and sample_velocity kernels run unchanged by the fixture generator (tests/golden/surface_field.npz),
against the oracle's restatement (CPU) and the GPU surfacer (mpm_surface_* through mpm_plugin_gb300.surface):
the normalised density field node for node and the velocity field sampled at 400 seeded points, within
1e-5. (The mesh itself comes from Warp's marching cubes, which is not in the reference's sources.)"""

from __future__ import annotations

import json

import numpy as np
import pytest
from _golden import GOLDEN

from oracle import surface as S

Z = np.load(GOLDEN / "surface_field.npz")
CASES = json.loads(str(Z["meta"]))["cases"]


def trilinear(field, pts):
    """Velocity field (dims + (3,)) at points in grid index units, the weights of field.py:68-88 in float64."""
    dims = np.array(field.shape[:3])
    i = np.clip(np.floor(pts).astype(int), 0, dims - 2)
    f = pts - i
    out = np.zeros((len(pts), 3))
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                w = (np.where(a, f[:, 0], 1 - f[:, 0]) * np.where(b, f[:, 1], 1 - f[:, 1]) *
                     np.where(c, f[:, 2], 1 - f[:, 2]))
                out += w[:, None] * field[i[:, 0] + a, i[:, 1] + b, i[:, 2] + c]
    return out


def _check(name, density, velocity):
    ref_d = Z[f"{name}_density"]
    assert density.shape == ref_d.shape
    assert np.abs(density - ref_d).max() <= 1e-5 * ref_d.max()
    got = trilinear(velocity.astype(np.float64), Z[f"{name}_sample_grid"].astype(np.float64))
    ref = Z[f"{name}_sample_vel"].astype(np.float64)
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref), np.linalg.norm(got - ref) / np.linalg.norm(ref)


@pytest.mark.parametrize("name", CASES)
def test_oracle_fields_match_reference(name):
    detail, smoothing, iso = Z[f"{name}_settings"]
    r = S.surface_particles(Z["positions"], Z["velocities"], float(Z["spacing"]), detail, smoothing, iso)
    _check(name, r["density"], r["velocity"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_fields_match_reference(name):
    from mpm_plugin_gb300.surface import SurfaceSettings, _surfacer, surface_particles

    detail, smoothing, iso = (float(v) for v in Z[f"{name}_settings"])
    surface_particles(Z["positions"], Z["velocities"], float(Z["spacing"]),
                      SurfaceSettings(detail=detail, smoothing=smoothing, iso=iso), device="cuda:0")
    dens, fld = _surfacer("cuda:0").read_field()
    _check(name, dens, fld[..., :3])

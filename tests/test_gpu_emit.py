"""Emitter volume sampling on the GPU against the reference's own outputs (tests/golden/geometry.npz, made by
running mpm_core.geometry.sample_mesh_volume) and against the oracle's restatement on further meshes:
bit-identical points in the same order."""

from __future__ import annotations

import json

import numpy as np
import pytest
from _golden import GOLDEN
from scenes import icosphere, rot_x, rot_z, scale, torus, translate, unit_cube_mesh

from oracle import geometry

pytestmark = pytest.mark.gpu


def test_matches_reference_fixtures():
    from mpm_plugin_gb300.emit import sample_mesh_volume

    z = np.load(GOLDEN / "geometry.npz")
    meta = json.loads(str(z["meta"]))
    for k, sm in enumerate(meta["samples"]):
        pts = sample_mesh_volume(z[f"sample{k}_verts"], z[f"sample{k}_tris"], sm["spacing"], sm["seed"])
        assert pts.dtype == np.float32
        np.testing.assert_array_equal(pts, z[f"sample{k}_points"])


def _meshes():
    cv, ct = unit_cube_mesh(centered=True)
    yield "cube on lattice columns", geometry.transform_points(translate(0.5, 0.5, 0.5) @ scale(0.25), cv), ct, 1 / 128
    yield "rotated slab", geometry.transform_points(translate(0.3, 0.6, 0.2) @ rot_z(30) @ rot_x(20) @ scale(0.3, 0.1, 0.05), cv), ct, 1 / 256
    sv, st = icosphere(0.12, 4, seed=3, jitter=0.05)
    yield "perturbed sphere", sv + np.float32([0.4, 0.5, 0.3]), st, 1 / 200
    tv, tt = torus(0.2, 0.05, 64, 16, seed=2, jitter=0.05)
    yield "torus (several crossings per column)", geometry.transform_points(translate(0.5, 0.5, 0.5) @ rot_x(60), tv), tt, 1 / 256


@pytest.mark.parametrize("seed", [0, [3, 7]])
def test_matches_oracle_on_harder_meshes(seed):
    from mpm_plugin_gb300.emit import sample_mesh_volume

    for name, v, t, spacing in _meshes():
        ref = geometry.sample_mesh_volume(v, t, spacing, seed)
        got = sample_mesh_volume(v, t, spacing, seed)
        assert len(ref) > 100, name
        np.testing.assert_array_equal(got, ref, err_msg=name)


def test_open_mesh_rejected():
    from mpm_plugin_gb300.emit import sample_mesh_volume

    cv, ct = unit_cube_mesh()
    with pytest.raises(ValueError, match="not closed"):
        sample_mesh_volume(cv, ct[:-1], 0.1, 0)

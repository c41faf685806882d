"""The seeded workloads bench.py measures (mpm_plugin_gb300.workloads): meshes, scene sizes, and the mesh
volumes sampled on the GPU against the oracle's restatement of the reference sampler (bit-identical)."""

from __future__ import annotations

import numpy as np
import pytest

from mpm_plugin_gb300 import workloads as w


def _closed_outward(verts, tris, centre):
    e = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), 1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    a, b, c = (verts[tris[:, k]].astype(np.float64) - centre for k in range(3))
    return bool((counts == 2).all()), bool(((np.cross(b - a, c - a) * (a + b + c)).sum(1) > 0).all())


@pytest.mark.parametrize("sub,tris", [(0, 20), (3, 1280), (4, 5120), (5, 20480)])
def test_geodesic_sphere(sub, tris):
    v, t = w.geodesic_sphere(2.0, sub)
    assert len(t) == tris and len(v) == tris // 2 + 2
    assert _closed_outward(v, t, 0.0) == (True, True)
    np.testing.assert_allclose(np.linalg.norm(v, axis=1), 2.0, rtol=1e-6)
    vj, tj = w.geodesic_sphere(2.0, sub, seed=3, jitter=0.03)
    assert np.array_equal(tj, t)
    r = np.linalg.norm(vj, axis=1) / 2.0
    assert r.min() >= 0.97 - 1e-6 and r.max() <= 1.03 + 1e-6 and r.std() > 0.005


def test_other_meshes_are_closed_and_outward():
    v, t = w.box_mesh((0.5, 0.4, 0.0), (0.65, 0.6, 0.4))
    assert len(t) == 12 and _closed_outward(v, t, np.float64([0.575, 0.5, 0.2])) == (True, True)
    v, t = w.torus(0.2, 0.05, 256, 40, seed=3, jitter=0.05)
    assert len(t) == 20480 and _closed_outward(v, t, 0.0)[0]
    v, t = w.cylinder(0.05, 0.02, 48)
    assert len(t) == 192 and _closed_outward(v, t, np.float64([0.0, 0.0, 0.01])) == (True, True)


def test_scene_sizes_and_domains():
    d, mats, pos = w.jelly_cube(64)
    assert len(pos) == 32768 and w.cell_size(d) == 1 / 64 and all(d.walls.values()) and len(d.walls) == 6
    d, mats, pile, (tv, tt), pose, emit = w.large_scene(256, 0.155)
    assert 7.4e6 < len(pile) < 7.5e6 and len(tt) == 20480 and w.cell_size(d) == 1 / 256
    specs = w.batched_scenes(seed=0, n_hi=2e6)
    n = [len(s[2]) for s in specs]
    assert len(specs) == 64 and min(n) >= 8e3 and max(n) <= 2.1e6 and 2.0e7 < sum(n) < 3.0e7
    assert {s[1][0].model for s in specs} == set(w.BATCH_MODELS)


@pytest.mark.gpu
def test_device_sampled_scene_equals_the_reference_sampler():
    """The mixed workload sampled on the GPU and by the oracle's restatement of the reference's sampler: the same
    points bit for bit (so bench.py's CPU arms, which sample on the CPU, time the same scene)."""
    from oracle import geometry

    _, _, gpu_groups, col = w.mixed_scene(128)
    _, _, cpu_groups, col2 = w.mixed_scene(128, sample=geometry.sample_mesh_volume)
    assert sum(len(g[0]) for g in gpu_groups) > 290_000
    for a, b in zip(gpu_groups, cpu_groups):
        np.testing.assert_array_equal(a[0], b[0])
        assert a[1:] == b[1:]
    np.testing.assert_array_equal(col[0], col2[0])

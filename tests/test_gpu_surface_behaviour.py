"""The reference's own surfacer tests (tests/test_surface_field.py) run against the GPU surfacer
(mpm_plugin_gb300.surface.surface_particles, the replacement of mpm_surface.field.surface_particles): shape,
closure, components, material at the floor, empty input, vertex velocity, detail, and the memory budget."""

from __future__ import annotations

import numpy as np
import pytest
from scenes import box_particles, sphere_particles

from oracle.geometry import mesh_is_closed

pytestmark = pytest.mark.gpu

SPACING = 0.005  # the particle helpers sample at dx / 2
DX = 0.01


def _settings(**kw):
    from mpm_plugin_gb300.surface import SurfaceSettings

    return SurfaceSettings(**kw)


def signed_volume(verts, tris):
    a, b, c = (verts[tris[:, k]].astype(np.float64) for k in range(3))
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6)


def components(tris):
    """Connected components of a triangle mesh (triangles joined through shared vertices)."""
    parent = {}

    def find(i):
        parent.setdefault(i, i)
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    for a, b, c in tris:
        ra, rb, rc = find(int(a)), find(int(b)), find(int(c))
        parent[rb] = ra
        parent[find(rc)] = ra
    return len({find(int(i)) for i in np.unique(tris)})


def mesh(p, vel=None, settings=None, **kw):
    from mpm_plugin_gb300.surface import surface_particles

    return surface_particles(p, np.zeros_like(p) if vel is None else vel, SPACING, settings or _settings(),
                             device="cuda:0", **kw)


def test_sphere_closed_outward_right_size():  # test_surface_field.py:37-43
    m = mesh(sphere_particles((0.5, 0.5, 0.5), 0.1, DX))
    assert mesh_is_closed(m.tris)
    vol = signed_volume(m.verts, m.tris)
    assert vol > 0 and vol == pytest.approx(4 / 3 * np.pi * 0.1 ** 3, rel=0.10)
    assert np.allclose(m.verts.mean(0), 0.5, atol=0.005)


def test_two_blobs_two_components():  # test_surface_field.py:46-49
    p = np.concatenate([sphere_particles((0.3, 0.5, 0.5), 0.05, DX), sphere_particles((0.7, 0.5, 0.5), 0.05, DX)])
    assert components(mesh(p).tris) == 2


def test_resting_on_floor_closed():  # test_surface_field.py:52-55: closes just below z = 0, no hole
    m = mesh(box_particles((0.4, 0.4, 0.0), (0.6, 0.6, 0.1), DX))
    assert mesh_is_closed(m.tris) and m.verts[:, 2].min() < 0.0


def test_empty():  # test_surface_field.py:58-61
    m = mesh(np.zeros((0, 3), np.float32))
    assert m.verts.shape == (0, 3) and m.tris.shape == (0, 3) and m.vel.shape == (0, 3)


def test_vertex_velocity():  # test_surface_field.py:64-68
    p = sphere_particles((0.5, 0.5, 0.5), 0.05, DX)
    m = mesh(p, vel=np.tile([1.0, 0, 0], (len(p), 1)).astype(np.float32))
    assert len(m.vel) == len(m.verts) and np.allclose(m.vel, [1.0, 0, 0], atol=1e-3)


def test_detail_increases_triangles():  # test_surface_field.py:71-75
    p = sphere_particles((0.5, 0.5, 0.5), 0.05, DX)
    assert len(mesh(p, settings=_settings(detail=2.0)).tris) > len(mesh(p, settings=_settings(detail=1.0)).tris)


def test_too_many_cells_raises():  # test_surface_field.py:78-81
    p = np.array([[0, 0, 0], [4, 4, 0.1]], np.float32)
    from mpm_plugin_gb300.surface import surface_particles

    with pytest.raises(ValueError, match="GPU memory"):
        surface_particles(p, np.zeros_like(p), 0.001, _settings(detail=2), device="cuda:0")


def test_memory_budget_counts_bytes():  # test_surface_field.py:84-88
    p = sphere_particles((0.5, 0.5, 0.5), 0.05, DX)
    with pytest.raises(ValueError, match="GPU memory"):
        mesh(p, max_bytes=1_000_000)

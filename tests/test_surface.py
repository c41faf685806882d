"""Surfacer host logic on the CPU: the marching-cubes case table (library vs an independent construction in
the oracle), the meshes it makes (closed, consistently wound outward), the rest density and the memory
budget check of surface_particles."""

from __future__ import annotations

import collections
import ctypes as C

import numpy as np
import pytest

from oracle import surface as S


def _device_table():
    from mpm_plugin_gb300 import _abi

    nt = np.zeros(256, np.int8)
    ed = np.zeros(256 * 36, np.int8)
    assert _abi.lib().mpm_mc_table(nt.ctypes.data_as(C.c_void_p), ed.ctypes.data_as(C.c_void_p)) == 0
    return [[tuple(int(x) for x in ed[m * 36 + 3 * t:m * 36 + 3 * t + 3]) for t in range(nt[m])] for m in range(256)]


def test_library_table_equals_the_independent_construction():
    dev, ref = _device_table(), S.mc_table()
    assert dev == ref
    assert max(len(t) for t in dev) == 5 and dev[0] == [] and dev[255] == []
    assert dev[1] == [(0, 4, 8)]  # one inside corner at the origin: x, y, z edges, normal towards (1, 1, 1)


def _manifold_errors(tris):
    cnt = collections.Counter()
    for a, b, c in tris:
        for e in ((a, b), (b, c), (c, a)):
            cnt[e] += 1
    return sum(1 for (a, b), n in cnt.items() if n != 1 or cnt.get((b, a), 0) != 1)


def _volume(verts, tris):
    v = verts[tris]
    return float(np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])).sum() / 6.0)


@pytest.mark.parametrize("seed", range(4))
def test_meshes_are_closed_and_wound_outward(seed):
    table = _device_table()
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(11, 11, 11)).astype(np.float32)
    f[0], f[-1], f[:, 0], f[:, -1], f[:, :, 0], f[:, :, -1] = -5, -5, -5, -5, -5, -5
    verts, tris = S.marching_cubes(f, np.float32(0.0), table)
    assert len(tris) > 100
    assert _manifold_errors(tris) == 0
    assert _volume(verts, tris) > 0


def test_sphere_field_gives_its_volume():
    g = np.indices((18, 18, 18)).transpose(1, 2, 3, 0) - 8.5
    verts, tris = S.marching_cubes((6.0 - np.linalg.norm(g, axis=-1)).astype(np.float32), np.float32(0.0))
    assert _manifold_errors(tris) == 0
    assert abs(_volume(verts, tris) / (4 / 3 * np.pi * 216) - 1) < 0.03


def test_rest_density_and_uniform_lattice_reads_one():
    from mpm_plugin_gb300.surface import rest_density

    assert rest_density(0.01, 0.04) == S.rest_density(0.01, 0.04)
    spacing = 0.02
    lat = (np.stack(np.meshgrid(*[np.arange(12)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * spacing
    out = S.surface_particles(lat.astype(np.float32), np.zeros_like(lat, np.float32), spacing, 1.0, 1.0, 0.35)
    d = out["density"]
    c = tuple(s // 2 for s in d.shape)
    assert abs(d[c] - 1.0) < 0.05  # field.py: a uniform lattice at `spacing` reads 1


def test_empty_input_gives_an_empty_mesh():
    from mpm_plugin_gb300.surface import SurfaceSettings, surface_particles

    m = surface_particles(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), 0.01, SurfaceSettings())
    assert m.verts.shape == (0, 3) and m.tris.shape == (0, 3) and m.tris.dtype == np.int32

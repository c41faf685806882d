"""Batches of independent scenes (mpm_batch_*, Gb300Batch) against the same scenes advanced one at a time.

A batch runs every kernel once for all scenes; each scene must come out as it does alone: the same
statistics per frame and the same state within the float-summation tolerance (P2G sums in a different order
when scenes share launches, as it does between any two runs).
"""

from __future__ import annotations

import numpy as np
import pytest
from _golden import rel_err
from scenes import ALL_WALLS, add, box_particles, domain, icosphere, preset, sphere_particles, translate, scale

from mpm_plugin_gb300.interface import ColliderGeometry, MeshData

pytestmark = pytest.mark.gpu


def _solver(d, mats):
    from mpm_plugin_gb300 import create

    return create(domain=d, materials=list(mats), gravity=(0.0, 0.0, -9.81), device="cuda:0")


def _scenes():
    """Four scenes of different sizes, grids, materials and colliders, one with an open side."""
    out = []
    d = domain(res=32)
    s = _solver(d, [preset("jelly")])
    add(s, box_particles((0.4, 0.4, 0.3), (0.6, 0.6, 0.5), d.dx, seed=1), 0, 0, (0.5, 0.0, 0.0))
    out.append(s)
    d = domain(res=64)
    s = _solver(d, [preset("sand_dry"), preset("snow_packed")])
    add(s, box_particles((0.3, 0.3, 0.0), (0.5, 0.5, 0.2), d.dx, seed=2), 0, 0)
    add(s, sphere_particles((0.7, 0.5, 0.3), 0.08, d.dx, seed=3), 1, 1, (-2.0, 0.0, 0.0))
    s.set_colliders([ColliderGeometry(MeshData(*icosphere(1.0, 3)), closed=True, friction=0.3)])
    xf = translate(0.5, 0.5, 0.45) @ scale(0.1)
    s.set_collider_transforms(xf[None], xf[None])
    out.append(s)
    d = domain(res=48, walls={**ALL_WALLS, "z-": False})
    s = _solver(d, [preset("whipped_cream")])
    add(s, box_particles((0.4, 0.4, 0.0), (0.6, 0.6, 0.2), d.dx, seed=4), 0, 0, (0.0, 0.0, -3.0))
    out.append(s)
    d = domain(res=16)
    out.append(_solver(d, [preset("jelly")]))  # empty scene
    return out


@pytest.mark.parametrize("sort_interval", [0, 4])
def test_batch_matches_scenes_alone(sort_interval):
    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.batch import Gb300Batch

    alone, batched = _scenes(), _scenes()
    for s in alone + batched:
        s.set_option(_abi.OPT_SORT_INTERVAL, sort_interval)
    batch = Gb300Batch(batched)
    batch.set_option(_abi.OPT_SORT_INTERVAL, sort_interval)
    fdt = [1 / 96, 1 / 120, 1 / 96, 1 / 96]
    for frame in range(3):
        st_alone = [s.advance(f) for s, f in zip(alone, fdt)]
        st_batch = batch.advance(fdt)
        for a, b in zip(st_alone, st_batch):
            assert a.substeps == b.substeps and a.removed == b.removed
            assert b.dt == pytest.approx(a.dt, rel=1e-3)
    assert batched[2].particle_count < len(box_particles((0.4, 0.4, 0.0), (0.6, 0.6, 0.2), 1 / 48, seed=4))
    for a, b in zip(alone, batched):
        sa, sb = a.save_state(), b.save_state()
        assert len(sa["x"]) == len(sb["x"])
        if len(sa["x"]) == 0:
            continue
        np.testing.assert_array_equal(sa["mat"], sb["mat"])
        np.testing.assert_array_equal(sa["emitter"], sb["emitter"])
        for k in ("x", "v", "F"):
            assert rel_err(sb[k], sa[k]) <= 1e-4, (k, rel_err(sb[k], sa[k]))
    batch.close()


def test_scene_leaves_batch_and_continues_alone():
    from mpm_plugin_gb300.batch import Gb300Batch

    scenes = _scenes()
    ref = _scenes()[0]
    batch = Gb300Batch(scenes)
    batch.advance(1 / 96)
    ref.advance(1 / 96)
    batch.remove(scenes[0])
    assert len(batch) == 3
    scenes[0].advance(1 / 96)
    ref.advance(1 / 96)
    batch.advance(1 / 96)
    assert rel_err(scenes[0].save_state()["x"], ref.save_state()["x"]) <= 1e-4
    scenes[1].close()  # a destroyed handle leaves its batch
    batch.advance(1 / 96)
    batch.close()
    scenes[2].advance(1 / 96)  # members stay usable after the batch is gone


def test_batch_errors():
    from mpm_plugin_gb300.batch import Gb300Batch

    s = _scenes()[0]
    b1, b2 = Gb300Batch([s]), Gb300Batch()
    with pytest.raises(ValueError, match="already belongs"):
        b2.add(s)
    with pytest.raises(ValueError, match="not in this batch"):
        b2.remove(s)
    with pytest.raises(ValueError, match="positive"):
        b1.advance(0.0)
    assert b2.advance(1 / 24) == []


def test_one_batched_substep_matches_the_scenes_alone_within_1e_5():
    """One substep per scene (a frame shorter than every scene's CFL step): the batched launches against each
    scene's own within 1e-5, the bar of the one-substep parity tests (C against |v| / dx)."""
    from mpm_plugin_gb300.batch import Gb300Batch

    alone, batched = _scenes(), _scenes()
    batch = Gb300Batch(batched)
    fdt = [2e-5, 1e-5, 2e-5, 2e-5]
    st_alone = [s.advance(f) for s, f in zip(alone, fdt)]
    st_batch = batch.advance(fdt)
    for a, b in zip(st_alone, st_batch):
        assert a.substeps == b.substeps
    assert [st.substeps for st in st_batch[:3]] == [1, 1, 1]
    for a, b in zip(alone, batched):
        sa, sb = a.save_state(), b.save_state()
        if len(sa["x"]) == 0:
            continue
        dx = 1.0 / a.domain.resolution
        gnorm = float(np.linalg.norm(sa["v"]) / dx)
        for k in ("x", "v", "C", "F", "Jp"):
            e = rel_err(sb[k], sa[k], floor=gnorm if k == "C" else 0.0)
            assert e <= 1e-5, (k, e)
    batch.close()

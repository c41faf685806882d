"""The reference's physical-outcome GPU tests, run against the gb300 backend.

Same scenes, steps and assertions as the reference suite (tests/test_warp_basic.py, test_warp_materials.py,
test_warp_colliders.py of the reference project), with the solver created as backend "gb300".
"""

from __future__ import annotations

import numpy as np
import pytest
from scenes import (ALL_WALLS, add, box_particles, domain, icosphere, plane_mesh, preset, preset_names, rot_x, rot_y,
                    scale, sphere_particles, translate, unit_cube_mesh)

from mpm_plugin_gb300.interface import ColliderGeometry, MeshData
from oracle.geometry import transform_points

pytestmark = pytest.mark.gpu


def make_solver(d, materials, gravity=(0.0, 0.0, -9.81)):
    from mpm_plugin_gb300 import create

    return create(domain=d, materials=list(materials), gravity=gravity, device="cuda:0")


def solver_with_box(d, material, lo, hi):
    s = make_solver(d, [material])
    add(s, box_particles(lo, hi, d.dx))
    return s


def run(s, frames, fps=24.0):
    for _ in range(frames):
        s.advance(1.0 / fps)


# --- test_warp_basic.py --------------------------------------------------------------------------------


def test_free_fall():  # test_warp_basic.py:12-21
    d = domain(res=64)
    s = make_solver(d, [preset("jelly")])
    p = box_particles((0.45, 0.45, 0.6), (0.55, 0.55, 0.7), d.dx)
    add(s, p)
    z0 = p[:, 2].mean()
    run(s, 6)
    assert z0 - s.get_particles().positions[:, 2].mean() == pytest.approx(0.5 * 9.81 * 0.25 ** 2, rel=0.02)


def test_rests_on_floor():  # test_warp_basic.py:24-33
    d = domain(res=64)
    s = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.0), (0.5, 0.5, 0.1))
    start = s.get_particles().positions.copy()
    run(s, 24)
    pos = s.get_particles().positions
    assert pos[:, 2].min() >= -0.25 * d.dx
    assert np.abs(pos - start).max() < 0.5 * d.dx


def test_non_cubic_domain():  # test_warp_basic.py:36-44
    d = domain((-0.5, -0.2, 0.0), (0.5, 0.05, 0.5), 64)
    assert d.grid_shape == (64, 16, 32)
    s = solver_with_box(d, preset("jelly"), (-0.05, -0.1, 0.3), (0.05, 0.0, 0.4))
    run(s, 24)
    pos = s.get_particles().positions
    assert pos[:, 2].min() >= -0.25 * d.dx and np.isfinite(pos).all()


def test_open_side_removes():  # test_warp_basic.py:47-52
    d = domain(res=32, walls={**ALL_WALLS, "z-": False})
    s = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.1), (0.6, 0.6, 0.2))
    removed = sum(s.advance(1 / 24).removed for _ in range(24))
    assert s.particle_count == 0 and removed > 0


def test_state_roundtrip():  # test_warp_basic.py:55-64
    d = domain(res=32)
    a = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.3), (0.6, 0.6, 0.5))
    a.advance(1 / 24)
    b = make_solver(d, [preset("jelly")])
    b.load_state(a.save_state())
    a.advance(1 / 24)
    b.advance(1 / 24)
    assert np.allclose(a.get_particles().positions, b.get_particles().positions, atol=1e-5)


def test_is_occupied():  # test_warp_basic.py:67-72
    d = domain(res=32)
    s = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.0), (0.6, 0.6, 0.2))
    s.advance(1 / 24)
    assert s.is_occupied(np.array([[0.5, 0.5, 0.1], [0.9, 0.9, 0.9]], np.float32)).tolist() == [True, False]


def test_nan_is_visible_in_positions():  # test_warp_basic.py:80-88
    d = domain(res=32)
    s = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.0), (0.5, 0.5, 0.1))
    state = s.save_state()
    state["v"][0] = np.nan
    s.load_state(state)
    s.advance(1 / 24)
    assert not np.isfinite(s.get_particles().positions).all()


@pytest.mark.parametrize("zmin", [0.0, 0.0100, 0.1326, 1.0359])
def test_wall_friction_independent_of_domain_placement(zmin):  # test_warp_basic.py:91-102
    a = np.radians(20)
    d = domain((0, 0, zmin), (1, 1, zmin + 1), 64, wall_friction=0.5)
    s = make_solver(d, [preset("whipped_cream")], gravity=(9.81 * np.sin(a), 0, -9.81 * np.cos(a)))
    p = box_particles((0.45, 0.45, zmin), (0.55, 0.55, zmin + 0.1), d.dx)
    add(s, p)
    run(s, 24)
    assert abs(s.get_particles().positions[:, 0].mean() - p[:, 0].mean()) < 0.005


# --- test_warp_materials.py ----------------------------------------------------------------------------


@pytest.mark.parametrize("name", preset_names())
def test_slab_at_rest(name):  # test_warp_materials.py:9-17
    d = domain((0, 0, 0), (0.5, 0.5, 0.5), 64)
    s = solver_with_box(d, preset(name), (0, 0, 0), (0.5, 0.5, 0.07))
    start = s.get_particles().positions.copy()
    run(s, 24)
    assert np.abs(s.get_particles().positions - start).max() < 0.5 * d.dx


def test_sand_column_collapses():  # test_warp_materials.py:20-28
    d = domain(res=64)
    s = solver_with_box(d, preset("sand_dry"), (0.44, 0.44, 0), (0.56, 0.56, 0.33))
    run(s, 48)
    pos = s.get_particles().positions
    assert pos[:, 2].max() < 0.6 * 0.33
    assert 0.12 < pos[:, 0].max() - 0.5 < 0.45


def test_cream_holds_shape():  # test_warp_materials.py:31-38
    d = domain(res=64)
    s = make_solver(d, [preset("whipped_cream")])
    add(s, sphere_particles((0.5, 0.5, 0.11), 0.11, d.dx))
    run(s, 48)
    z = s.get_particles().positions[:, 2]
    assert z.max() - z.min() > 0.5 * 0.22


def test_jelly_recovers():  # test_warp_materials.py:41-48
    d = domain(res=64)
    s = solver_with_box(d, preset("jelly"), (0.4, 0.4, 0.2), (0.6, 0.6, 0.4))
    run(s, 72)
    z = s.get_particles().positions[:, 2]
    assert z.max() - z.min() == pytest.approx(0.2, rel=0.15)


def test_mixed_materials_one_domain():  # test_warp_materials.py:51-58
    d = domain(res=64)
    s = make_solver(d, [preset("sand_dry"), preset("snow_packed")])
    add(s, box_particles((0.3, 0.3, 0), (0.5, 0.5, 0.1), d.dx, seed=0), 0, 0)
    add(s, box_particles((0.5, 0.5, 0), (0.7, 0.7, 0.1), d.dx, seed=1), 1, 1)
    run(s, 24)
    assert np.isfinite(s.get_particles().positions).all()


# --- test_warp_colliders.py ----------------------------------------------------------------------------

DOM = domain(res=64)
DX = DOM.dx


def points_in_box(pos, box_xf):
    local = transform_points(np.linalg.inv(box_xf), pos)
    half = 0.5 - 0.25 * DX / np.linalg.norm(box_xf[:3, :3], axis=0)
    return (np.abs(local) < half).all(axis=1)


def test_rests_on_open_plane():  # test_warp_colliders.py:47-55
    s = solver_with_box(DOM, preset("jelly"), (0.4, 0.4, 0.45), (0.6, 0.6, 0.55))
    s.set_colliders([ColliderGeometry(MeshData(*plane_mesh(0.8)), closed=False, friction=0.5)])
    xf = translate(0.5, 0.5, 0.3)
    s.set_collider_transforms(xf[None], xf[None])
    run(s, 36)
    zmin = s.get_particles().positions[:, 2].min()
    assert 0.3 - 0.25 * DX <= zmin <= 0.3 + 1.0 * DX


def test_scaled_box_collider():  # test_warp_colliders.py:58-65
    s = solver_with_box(DOM, preset("jelly"), (0.45, 0.45, 0.4), (0.55, 0.55, 0.5))
    s.set_colliders([ColliderGeometry(MeshData(*unit_cube_mesh(centered=True)), closed=True, friction=0.5)])
    xf = translate(0.5, 0.5, 0.0) @ scale(0.6, 0.6, 0.4)
    s.set_collider_transforms(xf[None], xf[None])
    run(s, 36)
    assert s.get_particles().positions[:, 2].min() == pytest.approx(0.2, abs=1.0 * DX)


@pytest.mark.parametrize("friction,slides", [(0.0, True), (1.0, False)])
def test_tilted_plane_friction(friction, slides):  # test_warp_colliders.py:68-77
    plane_xf = translate(0.5, 0.5, 0.3) @ rot_y(10)
    s = make_solver(DOM, [preset("whipped_cream")])
    local = box_particles((-0.05, -0.05, 0.25 * DX), (0.05, 0.05, 0.1), DX)
    add(s, transform_points(plane_xf, local))
    s.set_colliders([ColliderGeometry(MeshData(*plane_mesh(0.8)), closed=False, friction=friction)])
    s.set_collider_transforms(plane_xf[None], plane_xf[None])
    start = s.get_particles().positions.mean(0)
    run(s, 24)
    moved = np.linalg.norm(s.get_particles().positions.mean(0) - start)
    assert (moved > 0.05) if slides else (moved < 0.01)


def test_moving_box_clears_sand():  # test_warp_colliders.py:80-92
    s = solver_with_box(DOM, preset("sand_dry"), (0.1, 0.3, 0), (0.9, 0.7, 0.06))
    s.set_colliders([ColliderGeometry(MeshData(*unit_cube_mesh(centered=True)), closed=True, friction=0.5)])

    def box(x):
        return translate(x, 0.5, 0.05) @ scale(0.1, 0.5, 0.1)

    for f in range(24):
        s.set_collider_transforms(box(0.15 + 0.3 * f / 24)[None], box(0.15 + 0.3 * (f + 1) / 24)[None])
        s.advance(1 / 24)
    inside = points_in_box(s.get_particles().positions, box(0.45))
    assert inside.sum() <= 0.001 * s.particle_count


def test_spinning_sphere_does_not_disturb_sand():  # test_warp_colliders.py:102-121
    r = 0.12

    def displacement(deg_per_frame):
        def ball(deg):
            return translate(0.5, 0.5, 0.1) @ rot_x(deg) @ scale(r)

        s = solver_with_box(DOM, preset("sand_dry"), (0.25, 0.25, 0), (0.75, 0.75, 0.15))
        s.set_colliders([ColliderGeometry(MeshData(*icosphere(1.0, 5)), closed=True, friction=0.0)])
        s.set_collider_transforms(ball(0)[None], ball(0)[None])
        s.advance(1 / 24)
        start = s.get_particles().positions.copy()
        for f in range(6):
            s.set_collider_transforms(ball(deg_per_frame * f)[None], ball(deg_per_frame * (f + 1))[None])
            s.advance(1 / 24)
        return np.linalg.norm(s.get_particles().positions - start, axis=1).mean()

    assert displacement(90) < displacement(0) + 0.25 * DX


def test_unknown_model_and_material_errors():
    from mpm_plugin_gb300.interface import MaterialParams

    d = domain(res=16)
    s = make_solver(d, [preset("jelly")])
    with pytest.raises(ValueError, match="material id out of range"):
        s.add_particles(np.zeros((1, 3)), np.zeros((1, 3)), np.array([3]), np.zeros(1))
    bad = MaterialParams("x", "elastic", 1e5, 0.3, 1000.0)
    object.__setattr__(bad, "model", "plasma")
    with pytest.raises(NotImplementedError):
        make_solver(d, [bad])

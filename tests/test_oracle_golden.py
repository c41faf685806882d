"""The C oracle against the golden fixtures produced by the reference's own code (CPU only)."""

from __future__ import annotations

import json
from fractions import Fraction

import numpy as np
import pytest
from _golden import GOLDEN, SOLVER_CASES, Case, rel_err

from oracle import geometry
from oracle.oracle import OracleSolver, dp_alpha, lame, svd3

# FP32 oracle vs the reference's FP32 kernels: same operand order, so agreement is at rounding level.
# Multi-substep cases accumulate a little more (chaotic contact / plasticity decisions).
TOL = {"x": 1e-6, "v": 5e-6, "C": 2e-5, "F": 2e-6, "Jp": 1e-6}


def run_oracle(case: Case, precision="f32"):
    s = OracleSolver(case.domain, case.materials, case.gravity, case.ppc, precision=precision)
    s.load_state(case.state("in"))
    s.set_colliders(case.colliders())
    if case.transforms() is not None:
        s.set_collider_transforms(*case.transforms())
    a, extra = case.action, {}
    if a["kind"] == "substep":
        s.frame_dt = a["frame_dt"]
        for k in range(a.get("count", 1)):
            s.substep(a["dt"], a["s"][k] if isinstance(a["s"], list) else a["s"])
    elif a["kind"] == "advance":
        extra["stats"] = np.array([s.advance(f) for f in a["frame_dts"]], np.float64)
    elif a["kind"] == "occupied":
        extra["occupied"] = s.is_occupied(case.z["points"])
    return s.save_state(), extra


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_oracle_matches_reference(name):
    case = Case(name)
    out, extra = run_oracle(case)
    ref = case.state("out")
    assert len(out["x"]) == len(ref["x"])
    np.testing.assert_array_equal(out["mat"], ref["mat"])
    np.testing.assert_array_equal(out["emitter"], ref["emitter"])
    for k in ("x", "v"):
        np.testing.assert_array_equal(np.isfinite(out[k]), np.isfinite(ref[k]))
    for k, tol in TOL.items():
        assert rel_err(out[k], ref[k]) <= tol, (k, rel_err(out[k], ref[k]))
    if "stats" in extra:
        np.testing.assert_allclose(extra["stats"], case.z["stats"], rtol=1e-12)
    if "occupied" in extra:
        np.testing.assert_array_equal(extra["occupied"], case.z["occupied"])


def test_nan_stays_visible():
    out, _ = run_oracle(Case("nan_advance"))
    assert not np.isfinite(out["x"]).all()


@pytest.mark.parametrize("name", ["elastic_substep", "models_substep", "collider_sphere_substep"])
def test_fp64_oracle_close_to_fp32(name):
    """The FP64 instance of the same substep: FP32 rounding stays at the 1e-6..1e-4 level."""
    case = Case(name)
    o32, _ = run_oracle(case, "f32")
    o64, _ = run_oracle(case, "f64")
    for k in ("x", "F"):
        assert rel_err(o32[k], o64[k]) < 1e-5


def test_svd_convention():
    rng = np.random.default_rng(0)
    for A in [np.eye(3), np.diag([1.1, 0.95, -0.9]), np.diag([1e-6, 1, 1]), np.zeros((3, 3)),
              rng.normal(size=(3, 3)), np.array([[0, 1, 0], [1, 0, 0], [0, 0, 1.0]])]:
        U, s, V = svd3(A, "f64")
        np.testing.assert_allclose(U @ np.diag(s) @ V.T, A, atol=1e-12)
        assert np.linalg.det(U) == pytest.approx(1.0) and np.linalg.det(V) == pytest.approx(1.0)
        assert s[0] >= s[1] >= abs(s[2]) - 1e-15
        assert np.sign(s[2]) == np.sign(np.linalg.det(A)) or np.linalg.det(A) == 0


def test_geometry_restatement():
    z = np.load(GOLDEN / "geometry.npz")
    meta = json.loads(str(z["meta"]))
    for i, m in enumerate(z["mats"]):
        t, q, S = geometry.decompose_transform(m)
        np.testing.assert_allclose(t, z["t"][i], atol=1e-12)
        np.testing.assert_allclose(q, z["q"][i], atol=1e-12)
        np.testing.assert_allclose(S, z["S"][i], atol=1e-12)
    for k, i in enumerate(range(0, 24, 2)):
        for j, s in enumerate(meta["svals"]):
            np.testing.assert_array_equal(geometry.interpolate_transform(z["mats"][i], z["mats"][i + 1], s),
                                          z["interp"][k, j])
    for k, sm in enumerate(meta["samples"]):
        pts = geometry.sample_mesh_volume(z[f"sample{k}_verts"], z[f"sample{k}_tris"], sm["spacing"], sm["seed"])
        np.testing.assert_array_equal(pts, z[f"sample{k}_points"])


def test_emission_times():
    meta = json.loads(str(np.load(GOLDEN / "geometry.npz")["meta"]))
    emitters = [("inflow", 3, 8, 4), ("inflow", 2, 10, 3), ("fill", 1, 1, 1)]
    for f, expect in meta["emission_times"].items():
        got = [[str(s), e] for s, e in geometry.emission_times(emitters, int(f))]
        assert got == expect
    assert geometry.emission_times(emitters, 3)[0][0] == Fraction(1, 3)


def test_material_constants():
    from _golden import material_from_dict

    meta = json.loads(str(np.load(GOLDEN / "geometry.npz")["meta"]))
    for pid, p in meta["presets"].items():
        m = material_from_dict(p["material"])
        assert lame(m) == (p["mu"], p["lam"])
        assert dp_alpha(m.friction_angle_deg) == p["alpha"]


def test_domain_constants():
    """dx and the grid shape the reference derives from a domain, against the oracle's restatement and the
    library's own (mpm_domain_grid_dims: grid shape + 6 padding nodes), which needs no GPU."""
    from _golden import Domain

    from mpm_plugin_gb300.interface import domain_grid_dims

    meta = json.loads(str(np.load(GOLDEN / "geometry.npz")["meta"]))
    for d in meta["domains"]:
        dom = Domain(tuple(d["min"]), tuple(d["max"]), d["resolution"])
        assert dom.dx == d["dx"] and list(dom.grid_shape) == d["grid_shape"]
        assert list(domain_grid_dims(dom)) == [s + 6 for s in d["grid_shape"]]

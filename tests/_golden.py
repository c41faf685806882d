"""Loading the golden fixtures (written by tests/golden/make_golden.py from the reference's own code)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from dataclasses import fields

from mpm_plugin_gb300.interface import Domain as _Domain
from mpm_plugin_gb300.interface import MaterialParams
from oracle.oracle import domain_dx, domain_grid_shape

WALL_SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")


class Domain(_Domain):
    """The interface's Domain (mpm_core's, or the data-only stand-in) with dx and grid_shape from the oracle's
    restatement of mpm_core/scene.py:60-67, so tests read the same either way; every wall side is listed."""

    def __init__(self, min, max, resolution, walls=None, wall_friction=0.5):  # noqa: A002
        super().__init__(tuple(min), tuple(max), resolution, {**{s: True for s in WALL_SIDES}, **(walls or {})},
                         wall_friction)

    @property
    def dx(self) -> float:
        return domain_dx(self)

    @property
    def grid_shape(self) -> tuple[int, int, int]:
        return domain_grid_shape(self)


def material_from_dict(d: dict) -> MaterialParams:
    """A MaterialParams from a preset's material table (keys that are not fields are ignored)."""
    known = {f.name for f in fields(MaterialParams)}
    return MaterialParams(**{k: v for k, v in d.items() if k in known})

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE_KEYS = ("x", "v", "C", "F", "Jp", "mat", "emitter")
SOLVER_CASES = ["elastic_substep", "models_substep", "models_3substeps", "walls_substep", "walls_advance",
                "collider_box_substep", "collider_plane_substep", "collider_sphere_substep", "nan_advance",
                "jelly_advance", "occupied"]


class Case:
    def __init__(self, name: str):
        self.name = name
        self.z = np.load(GOLDEN / f"{name}.npz")
        self.meta = json.loads(str(self.z["meta"]))
        d = self.meta["domain"]
        self.domain = Domain(tuple(d["min"]), tuple(d["max"]), d["resolution"], d["walls"], d["wall_friction"])
        self.materials = [material_from_dict(m) for m in self.meta["materials"]]
        self.gravity = tuple(self.meta["gravity"])
        self.ppc = self.meta["ppc"]
        self.action = self.meta["action"]

    def state(self, prefix: str) -> dict:
        return {k: self.z[f"{prefix}_{k}"] for k in STATE_KEYS}

    def colliders(self):
        """[(verts, tris, closed, friction), ...]"""
        return [(self.z[f"col{i}_verts"], self.z[f"col{i}_tris"], c["closed"], c["friction"])
                for i, c in enumerate(self.meta["colliders"])]

    def transforms(self):
        if "xf_start" in self.z:
            return self.z["xf_start"], self.z["xf_end"]
        return None


def rel_err(a, b, floor: float = 0.0) -> float:
    """Norm-wise relative error ||a - b|| / max(||b||, floor) over the finite entries."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    fin = np.isfinite(a) & np.isfinite(b)
    den = max(np.linalg.norm(b[fin]), floor)
    return float(np.linalg.norm((a - b)[fin]) / den) if den > 0 else float(np.linalg.norm((a - b)[fin]))

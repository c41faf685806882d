"""The solver interface this backend plugs into, and the scene records it consumes.

When the reference's ``mpm_core`` package is importable, its own classes are used, so ``Gb300Solver`` is a
real ``mpm_core.solver.Solver`` and registers with ``mpm_core.backends``. Where it is not installed (a bare
GPU host), records with the same names, fields and validation are defined here so the backend still works:

  ParticleData, AdvanceStats, ColliderGeometry, Solver   mpm_core/solver.py:15-82
  Domain (dx, grid_shape), MeshData                      mpm_core/scene.py:36-77
  MaterialParams (validation, lame)                      mpm_core/materials.py:24-59
"""

from __future__ import annotations

import math
from abc import ABC, abstractmethod
from collections.abc import Sequence
from dataclasses import asdict, dataclass, field, fields

import numpy as np

try:  # the reference package, when present, is the interface
    from mpm_core.materials import MaterialParams
    from mpm_core.scene import Domain, MeshData
    from mpm_core.solver import AdvanceStats, ColliderGeometry, ParticleData, Solver

    HAVE_MPM_CORE = True
except ImportError:  # same records, defined locally
    HAVE_MPM_CORE = False

    MODELS = ("elastic", "von_mises", "drucker_prager", "snow")
    WALL_SIDES = ("x-", "x+", "y-", "y+", "z-", "z+")

    @dataclass(frozen=True)
    class MaterialParams:  # type: ignore[no-redef]
        name: str
        model: str
        youngs_modulus: float
        poisson_ratio: float
        density: float
        yield_stress: float = 0.0
        friction_angle_deg: float = 0.0
        hardening: float = 0.0
        critical_compression: float = 0.0
        critical_stretch: float = 0.0
        max_hardening: float = 5.0

        def __post_init__(self):
            if self.model not in MODELS:
                raise ValueError(f"unknown material model {self.model!r}, expected one of {MODELS}")
            if not self.youngs_modulus > 0:
                raise ValueError("youngs_modulus must be > 0")
            if not 0 <= self.poisson_ratio < 0.5:
                raise ValueError("poisson_ratio must be in [0, 0.5)")
            if not self.density > 0:
                raise ValueError("density must be > 0")

        def lame(self) -> tuple[float, float]:
            e, nu = self.youngs_modulus, self.poisson_ratio
            return e / (2 * (1 + nu)), e * nu / ((1 + nu) * (1 - 2 * nu))

        def to_dict(self) -> dict:
            return asdict(self)

        @classmethod
        def from_dict(cls, d: dict) -> MaterialParams:
            known = {f.name for f in fields(cls)}
            return cls(**{k: v for k, v in d.items() if k in known})

    def _all_walls() -> dict[str, bool]:
        return {side: True for side in WALL_SIDES}

    @dataclass
    class Domain:  # type: ignore[no-redef]
        min: tuple[float, float, float]
        max: tuple[float, float, float]
        resolution: int
        walls: dict[str, bool] = field(default_factory=_all_walls)
        wall_friction: float = 0.5

        def __post_init__(self):
            self.min = tuple(float(x) for x in self.min)
            self.max = tuple(float(x) for x in self.max)
            if any(b <= a for a, b in zip(self.min, self.max)):
                raise ValueError("domain max must be greater than min on every axis")
            if self.resolution < 4:
                raise ValueError("domain resolution must be at least 4")
            self.walls = {**_all_walls(), **self.walls}
            unknown = set(self.walls) - set(WALL_SIDES)
            if unknown:
                raise ValueError(f"unknown wall sides {sorted(unknown)}")

        @property
        def size(self) -> tuple[float, float, float]:
            return tuple(b - a for a, b in zip(self.min, self.max))

        @property
        def dx(self) -> float:
            return max(self.size) / self.resolution

        @property
        def grid_shape(self) -> tuple[int, int, int]:
            return tuple(max(1, math.ceil(s / self.dx - 1e-6)) for s in self.size)

    @dataclass
    class MeshData:  # type: ignore[no-redef]
        verts: np.ndarray
        tris: np.ndarray

        def __post_init__(self):
            self.verts = np.asarray(self.verts, np.float32).reshape(-1, 3)
            self.tris = np.asarray(self.tris, np.int32).reshape(-1, 3)

    @dataclass
    class ParticleData:  # type: ignore[no-redef]
        positions: np.ndarray
        velocities: np.ndarray
        material_ids: np.ndarray
        emitter_ids: np.ndarray

    @dataclass
    class AdvanceStats:  # type: ignore[no-redef]
        substeps: int
        dt: float
        removed: int

    @dataclass
    class ColliderGeometry:  # type: ignore[no-redef]
        mesh: MeshData
        closed: bool
        friction: float

    class Solver(ABC):  # type: ignore[no-redef]
        def __init__(self, domain: Domain, materials: Sequence[MaterialParams], gravity, particles_per_cell: int = 8,
                     device: str | None = None):
            self.domain = domain
            self.materials = list(materials)
            self.gravity = tuple(float(g) for g in gravity)
            self.particles_per_cell = particles_per_cell
            self.device = device

        @abstractmethod
        def add_particles(self, positions, velocities, material_ids, emitter_ids) -> None: ...

        @abstractmethod
        def set_colliders(self, colliders) -> None: ...

        @abstractmethod
        def set_collider_transforms(self, start, end) -> None: ...

        @abstractmethod
        def advance(self, frame_dt: float) -> AdvanceStats: ...

        @property
        @abstractmethod
        def particle_count(self) -> int: ...

        @abstractmethod
        def get_particles(self) -> ParticleData: ...

        @abstractmethod
        def is_occupied(self, points) -> np.ndarray: ...

        @abstractmethod
        def save_state(self) -> dict: ...

        @abstractmethod
        def load_state(self, state: dict) -> None: ...

__all__ = ["HAVE_MPM_CORE", "AdvanceStats", "ColliderGeometry", "Domain", "MaterialParams", "MeshData",
           "ParticleData", "Solver"]

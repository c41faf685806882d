"""The solver interface this backend plugs into, and the scene records it consumes.

The interface is the reference's own: when ``mpm_core`` is importable, its classes are used, so
``Gb300Solver`` is a real ``mpm_core.solver.Solver`` and registers with ``mpm_core.backends``:

  ParticleData, AdvanceStats, ColliderGeometry, Solver   mpm_core/solver.py:15-82
  Domain, MeshData                                       mpm_core/scene.py:36-77
  MaterialParams                                         mpm_core/materials.py:24-59

Where ``mpm_core`` is not installed, plain records with the same names and fields stand in, so the backend can
be driven directly (``HAVE_MPM_CORE`` is then False and nothing is registered). They carry data only: no
validation, no derived quantities. The library validates what it is given (domain, materials, arrays) at the
C boundary, and the grid that a domain implies comes from it (``domain_grid_dims``).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

try:  # the reference package, when present, is the interface
    from mpm_core.materials import MaterialParams
    from mpm_core.scene import Domain, MeshData
    from mpm_core.solver import AdvanceStats, ColliderGeometry, ParticleData, Solver

    HAVE_MPM_CORE = True
except ImportError:  # data-only stand-ins with the interface's names and fields
    HAVE_MPM_CORE = False

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

    @dataclass
    class Domain:  # type: ignore[no-redef]
        min: tuple[float, float, float]
        max: tuple[float, float, float]
        resolution: int
        walls: dict[str, bool] = field(default_factory=dict)  # a side not listed is a wall
        wall_friction: float = 0.5

    @dataclass
    class MeshData:  # type: ignore[no-redef]
        verts: np.ndarray
        tris: np.ndarray

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

    class Solver:  # type: ignore[no-redef]
        """Base of a backend: keeps the constructor's arguments."""

        def __init__(self, domain, materials, gravity, particles_per_cell: int = 8, device: str | None = None):
            self.domain = domain
            self.materials = list(materials)
            self.gravity = tuple(float(g) for g in gravity)
            self.particles_per_cell = particles_per_cell
            self.device = device


def domain_desc(domain):
    """The C descriptor of a domain (include/mpm_gb300.h MpmDomainDesc); a side missing from ``walls`` is a
    wall, as the reference's Domain fills it in."""
    from mpm_plugin_gb300 import _abi

    d = _abi.MpmDomainDesc()
    walls = getattr(domain, "walls", None) or {}
    for a, ax in enumerate("xyz"):
        d.min[a] = float(domain.min[a])
        d.max[a] = float(domain.max[a])
        d.wall_lo[a] = int(bool(walls.get(f"{ax}-", True)))
        d.wall_hi[a] = int(bool(walls.get(f"{ax}+", True)))
    d.resolution = int(domain.resolution)
    d.wall_friction = float(domain.wall_friction)
    return d


def domain_grid_dims(domain) -> tuple[int, int, int]:
    """Nodes per axis of the padded grid the library builds for ``domain`` (grid shape + 6)."""
    import ctypes as C

    from mpm_plugin_gb300 import _abi

    dims = (C.c_int32 * 3)()
    _abi.check(_abi.lib().mpm_domain_grid_dims(C.byref(domain_desc(domain)), dims))
    return tuple(int(v) for v in dims)


__all__ = ["HAVE_MPM_CORE", "AdvanceStats", "ColliderGeometry", "Domain", "MaterialParams", "MeshData",
           "ParticleData", "Solver", "domain_desc", "domain_grid_dims"]

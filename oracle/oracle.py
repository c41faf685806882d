"""ctypes driver of the C oracle and an oracle solver with the reference's host logic. TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py import this module, and only as
the checker (or the timed CPU baseline). The product never imports it.

``OracleSolver`` restates the host side of mpm_core/backends/warp/solver.py around the C kernels:
grid/padding/wall-node set-up (37-53), material tables (56-71), particle append (100-125), collider pose
decomposition (154-172), CFL time step (176-185), substep order (187-211), advance (213-220), removal of
escaped particles (222-240) and occupancy queries (244-255).
"""

from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from oracle import build as _build
from oracle import geometry

PAD = 3
CFL = 0.4
COLLIDER_THICKNESS = 2.0
MODEL_IDS = {"elastic": 0, "von_mises": 1, "drucker_prager": 2, "snow": 3}
STATE_KEYS = ("x", "v", "C", "F", "Jp", "mat", "emitter")


class OrcDomain(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("wall_lo_node", C.c_int * 3), ("wall_hi_node", C.c_int * 3),
                ("lo_on", C.c_int * 3), ("hi_on", C.c_int * 3), ("origin", C.c_double * 3), ("dx", C.c_double),
                ("inv_dx", C.c_double), ("p_vol", C.c_double), ("gravity", C.c_double * 3),
                ("wall_friction", C.c_double), ("wall_lo", C.c_double * 3), ("wall_hi", C.c_double * 3),
                ("clamp_lo", C.c_double * 3), ("clamp_hi", C.c_double * 3), ("thickness", C.c_double),
                ("band", C.c_double)]


class OrcMaterial(C.Structure):
    _fields_ = [("model", C.c_int), ("mu", C.c_double), ("lam", C.c_double), ("yield_stress", C.c_double),
                ("alpha", C.c_double), ("hardening", C.c_double), ("max_hardening", C.c_double),
                ("crit_c", C.c_double), ("crit_s", C.c_double), ("density", C.c_double)]


class OrcCollider(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("closed", C.c_int), ("friction", C.c_double), ("margin", C.c_double),
                ("aabb_lo", C.c_double * 3), ("aabb_hi", C.c_double * 3), ("t0", C.c_double * 3),
                ("t1", C.c_double * 3), ("q0", C.c_double * 4), ("q1", C.c_double * 4), ("S0", C.c_double * 9),
                ("S1", C.c_double * 9)]


_libs: dict[str, C.CDLL] = {}


def lib(precision: str = "f32") -> C.CDLL:
    if precision not in _libs:
        _build.build()
        L = C.CDLL(str(_build.lib_path(precision)))
        R = C.c_float if precision == "f32" else C.c_double
        P = C.c_void_p
        L.orc_mesh_new.restype = P
        L.orc_mesh_new.argtypes = [C.c_int, P, C.c_int, P]
        L.orc_mesh_free.argtypes = [P]
        L.orc_mesh_query.restype = C.c_int
        L.orc_mesh_query.argtypes = [P, P, P, P, P, P]
        L.orc_svd3.argtypes = [P, P, P, P]
        L.orc_substep.argtypes = [P, P, C.c_int, P, C.c_int, P, P, P, P, P, P, R, R, R, P, C.c_int]
        L.orc_p2g.argtypes = [P, P, C.c_int, P, P, P, P, P, P, R, P, C.c_int]
        L.orc_grid_update.argtypes = [P, R, P, C.c_int]
        L.orc_collider_pose.argtypes = [P, R, R, P, P, P]
        L.orc_max_speed.restype = R
        L.orc_max_speed.argtypes = [C.c_int, P]
        L.orc_scatter_volume.argtypes = [P, C.c_int, P, P]
        L.orc_query_fill.argtypes = [P, C.c_int, P, P, P]
        _libs[precision] = L
    return _libs[precision]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def domain_dx(domain) -> float:
    """mpm_core/scene.py:60-62: the longest side over the resolution."""
    size = [b - a for a, b in zip(domain.min, domain.max)]
    return max(size) / domain.resolution


def domain_grid_shape(domain) -> tuple[int, int, int]:
    """mpm_core/scene.py:64-67."""
    dx = domain_dx(domain)
    return tuple(max(1, math.ceil((b - a) / dx - 1e-6)) for a, b in zip(domain.min, domain.max))


def make_domain(domain, gravity, ppc: int) -> OrcDomain:
    """Host constants of warp/solver.py:37-53 (float64 here, rounded to REAL inside the oracle)."""
    d = OrcDomain()
    dx = domain_dx(domain)
    dims = [s + 2 * PAD for s in domain_grid_shape(domain)]
    origin = np.asarray(domain.min, np.float64) - PAD * dx
    for a, ax in enumerate("xyz"):
        d.dims[a] = dims[a]
        d.origin[a] = origin[a]
        d.lo_on[a] = int(domain.walls[f"{ax}-"])
        d.hi_on[a] = int(domain.walls[f"{ax}+"])
        d.wall_lo[a] = domain.min[a]
        d.wall_hi[a] = domain.max[a]
        d.clamp_lo[a] = origin[a] + dx
        d.clamp_hi[a] = origin[a] + (dims[a] - 2) * dx
        d.wall_lo_node[a] = int(math.floor((domain.min[a] - origin[a]) / dx + 1e-3))
        d.wall_hi_node[a] = int(math.ceil((domain.max[a] - origin[a]) / dx - 1e-3))
        d.gravity[a] = float(gravity[a])
    d.dx = dx
    d.inv_dx = 1.0 / dx
    d.p_vol = dx ** 3 / ppc
    d.wall_friction = domain.wall_friction
    d.thickness = COLLIDER_THICKNESS * dx
    d.band = dx
    return d


def lame(m) -> tuple[float, float]:
    """mpm_core/materials.py:48-51."""
    e, nu = m.youngs_modulus, m.poisson_ratio
    return e / (2 * (1 + nu)), e * nu / ((1 + nu) * (1 - 2 * nu))


def dp_alpha(friction_angle_deg: float) -> float:
    """warp/solver.py:263-265."""
    s = math.sin(math.radians(friction_angle_deg))
    return math.sqrt(2 / 3) * 2 * s / (3 - s)


def make_materials(materials):
    arr = (OrcMaterial * max(1, len(materials)))()
    for i, m in enumerate(materials):
        mu, lam = lame(m)
        arr[i] = OrcMaterial(MODEL_IDS[m.model], mu, lam, m.yield_stress, dp_alpha(m.friction_angle_deg),
                             m.hardening, m.max_hardening, m.critical_compression, m.critical_stretch, m.density)
    return arr


def wave_speeds(materials) -> np.ndarray:
    """P-wave speed per material with worst-case snow hardening, warp/solver.py:59-62."""
    out = []
    for m in materials:
        mu, lam = lame(m)
        out.append(math.sqrt((lam + 2 * mu) * (m.max_hardening if m.model == "snow" else 1.0) / m.density))
    return np.array(out, np.float64)


class OracleMesh:
    def __init__(self, verts, tris, precision="f32"):
        self.verts = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 3))
        self.tris = np.ascontiguousarray(np.asarray(tris, np.int32).reshape(-1, 3))
        self._lib = lib(precision)
        self.handle = self._lib.orc_mesh_new(len(self.verts), _ptr(self.verts), len(self.tris), _ptr(self.tris))

    def query(self, p):
        p = np.asarray(p, np.float64)
        out = np.zeros(4)
        f = self._lib.orc_mesh_query(self.handle, _ptr(p), _ptr(out[0:1]), _ptr(out[1:2]), _ptr(out[2:3]),
                                     _ptr(out[3:4]))
        return f, out[0], out[1], out[2], out[3]

    def __del__(self):
        try:
            self._lib.orc_mesh_free(self.handle)
        except Exception:
            pass


class OracleSolver:
    """The reference WarpSolver's behaviour on the CPU, kernels in C (REAL = float32 or float64)."""

    def __init__(self, domain, materials, gravity, particles_per_cell: int = 8, precision: str = "f32",
                 threads: int = 1):
        self.domain = domain
        self.materials = list(materials)
        for m in self.materials:
            if m.model not in MODEL_IDS:
                raise NotImplementedError(f"material model {m.model!r} is not supported")
        self.gravity = tuple(float(g) for g in gravity)
        self.ppc = particles_per_cell
        self.precision = precision
        self.threads = threads
        self.lib = lib(precision)
        self.real = np.float32 if precision == "f32" else np.float64
        self.dx = domain_dx(domain)
        self.d = make_domain(domain, self.gravity, particles_per_cell)
        self.dims = tuple(self.d.dims)
        self.mats = make_materials(self.materials)
        self.wave = wave_speeds(self.materials)
        self.grid = np.zeros(self.dims + (4,), self.real)
        self.meshes: list[OracleMesh] = []
        self.cols = (OrcCollider * 1)()
        self.n_col = 0
        self.frame_dt = 1.0
        self._set({"x": np.zeros((0, 3)), "v": np.zeros((0, 3)), "C": np.zeros((0, 3, 3)), "F": np.zeros((0, 3, 3)),
                   "Jp": np.zeros(0), "mat": np.zeros(0, np.int32), "emitter": np.zeros(0, np.int32)})

    # -- state (warp/solver.py:82-138)
    def _set(self, s):
        """Copies of the given arrays (the kernels update the state in place; the caller's arrays stay as
        they were, as the reference's state upload leaves them)."""
        r = self.real
        self.x = np.array(s["x"], r, order="C").reshape(-1, 3)
        self.v = np.array(s["v"], r, order="C").reshape(-1, 3)
        self.C = np.array(s["C"], r, order="C").reshape(-1, 3, 3)
        self.F = np.array(s["F"], r, order="C").reshape(-1, 3, 3)
        self.Jp = np.array(s["Jp"], r, order="C").reshape(-1)
        self.mat = np.array(s["mat"], np.int32, order="C").reshape(-1)
        self.emitter = np.array(s["emitter"], np.int32, order="C").reshape(-1)
        self.present = np.unique(self.mat)

    def load_state(self, s):
        self._set(s)

    def save_state(self) -> dict:
        return {k: getattr(self, k).copy() for k in STATE_KEYS}

    @property
    def particle_count(self) -> int:
        return len(self.x)

    def add_particles(self, pos, vel, mat, emitter):
        n = len(pos)
        if n == 0:
            return
        mat = np.asarray(mat, np.int32)
        if mat.min() < 0 or mat.max() >= len(self.materials):
            raise ValueError("material id out of range")
        new = {"x": np.asarray(pos).reshape(n, 3), "v": np.asarray(vel).reshape(n, 3), "C": np.zeros((n, 3, 3)),
               "F": np.tile(np.eye(3), (n, 1, 1)), "Jp": np.ones(n), "mat": mat, "emitter": np.asarray(emitter)}
        cur = self.save_state()
        self._set({k: np.concatenate([cur[k], np.asarray(new[k], cur[k].dtype)]) for k in STATE_KEYS})

    # -- colliders (warp/solver.py:142-172)
    def set_colliders(self, colliders):
        """colliders: sequence of (verts, tris, closed, friction)."""
        self.meshes = [OracleMesh(v, t, self.precision) for v, t, _, _ in colliders]
        self.col_info = [(bool(c), float(f), np.asarray(v, np.float32).reshape(-1, 3)) for v, _, c, f in colliders]
        self.n_col = len(colliders)
        self.cols = (OrcCollider * max(1, self.n_col))()
        eye = np.tile(np.eye(4, dtype=np.float32), (self.n_col, 1, 1))
        self.set_collider_transforms(eye, eye)

    def set_collider_transforms(self, start, end):
        start = np.asarray(start, np.float32).reshape(-1, 4, 4)
        end = np.asarray(end, np.float32).reshape(-1, 4, 4)
        if len(start) != self.n_col or len(end) != self.n_col:
            raise ValueError(f"expected {self.n_col} collider transforms")
        for c, (a, b) in enumerate(zip(start, end)):
            closed, fric, verts = self.col_info[c]
            t0, q0, S0 = geometry.decompose_transform(a)
            t1, q1, S1 = geometry.decompose_transform(b)
            if np.dot(q0, q1) < 0:
                q1 = -q1
            inv_scale = max(1.0 / max(np.linalg.svd(m[:3, :3], compute_uv=False).min(), 1e-12) for m in (a, b))
            col = self.cols[c]
            col.mesh = self.meshes[c].handle
            col.closed = int(closed)
            col.friction = fric
            col.margin = 3.0 * self.dx * inv_scale
            lo, hi = verts.min(0), verts.max(0)
            for k in range(3):
                col.aabb_lo[k] = float(lo[k])
                col.aabb_hi[k] = float(hi[k])
                col.t0[k] = t0[k]
                col.t1[k] = t1[k]
            for k in range(4):
                col.q0[k] = q0[k]
                col.q1[k] = q1[k]
            for k in range(9):
                col.S0[k] = S0.ravel()[k]
                col.S1[k] = S1.ravel()[k]

    # -- stepping (warp/solver.py:176-220)
    def choose_dt(self, frame_dt: float):
        vmax = float(self.lib.orc_max_speed(len(self.v), _ptr(self.v)))
        if not math.isfinite(vmax):
            vmax = 0.0
        c = float(self.wave[self.present].max())
        dt = min(CFL * self.dx / (c + vmax), frame_dt)
        steps = math.ceil(frame_dt / dt - 1e-9)
        return frame_dt / steps, steps

    def substep(self, dt: float, s: float):
        n = len(self.x)
        self.lib.orc_substep(C.byref(self.d), self.mats, self.n_col, self.cols, n, _ptr(self.x), _ptr(self.v),
                             _ptr(self.C), _ptr(self.F), _ptr(self.Jp), _ptr(self.mat), dt, s, 1.0 / self.frame_dt,
                             _ptr(self.grid), self.threads)

    def advance(self, frame_dt: float):
        if len(self.x) == 0:
            return 0, frame_dt, 0
        self.frame_dt = frame_dt
        dt, steps = self.choose_dt(frame_dt)
        for k in range(steps):
            self.substep(dt, (k + 1) / steps)
        return steps, dt, self.remove_escaped()

    def remove_escaped(self) -> int:
        dom = self.domain
        out = np.zeros(len(self.x), bool)
        any_open = False
        for a, ax in enumerate("xyz"):
            if not dom.walls[f"{ax}-"]:
                any_open = True
                out |= self.x[:, a] < self.real(dom.min[a] - self.dx)
            if not dom.walls[f"{ax}+"]:
                any_open = True
                out |= self.x[:, a] > self.real(dom.max[a] + self.dx)
        if not any_open:
            return 0
        removed = int(out.sum())
        if removed:
            s = self.save_state()
            self._set({k: v[~out] for k, v in s.items()})
        return removed

    def collider_pose(self, c: int, s: float):
        """(M, M^-1, dM/dt) of collider c at substep fraction s, each 3x4 (colliders.py:30-37, 68-74)."""
        out = [np.zeros((4, 4), self.real) for _ in range(3)]
        self.lib.orc_collider_pose(C.byref(self.cols[c]), s, 1.0 / self.frame_dt, *(_ptr(a) for a in out))
        return tuple(a[:3] for a in out)

    def is_occupied(self, points) -> np.ndarray:
        pts = np.ascontiguousarray(np.asarray(points, self.real).reshape(-1, 3))
        if len(pts) == 0:
            return np.zeros(0, bool)
        vol = np.zeros(self.dims, self.real)
        self.lib.orc_scatter_volume(C.byref(self.d), len(self.x), _ptr(self.x), _ptr(vol))
        out = np.zeros(len(pts), np.uint8)
        self.lib.orc_query_fill(C.byref(self.d), len(pts), _ptr(pts), _ptr(vol), _ptr(out))
        return out.astype(bool)


def svd3(A, precision="f32"):
    r = np.float32 if precision == "f32" else np.float64
    A = np.ascontiguousarray(np.asarray(A, r).reshape(3, 3))
    U, s, V = np.zeros((3, 3), r), np.zeros(3, r), np.zeros((3, 3), r)
    lib(precision).orc_svd3(_ptr(A), _ptr(U), _ptr(s), _ptr(V))
    return U, s, V


ROOT = Path(__file__).resolve().parent.parent

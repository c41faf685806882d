"""Gb300Solver: the reference's solver interface (numpy in, numpy out) over the sm_103a kernels.

Drop-in for ``mpm_core.backends.warp.solver.WarpSolver`` (mpm_core/backends/warp/solver.py:26-255): the same
constructor arguments, methods, array shapes and dtypes, the same exceptions for the same mistakes, and the
same particle order. All device memory belongs to the library handle; numpy inputs are copied.
"""

from __future__ import annotations

import ctypes as C
from collections.abc import Sequence

import numpy as np

from mpm_plugin_gb300 import _abi
from mpm_plugin_gb300.interface import AdvanceStats, ColliderGeometry, ParticleData, Solver, domain_desc

STATE_KEYS = ("x", "v", "C", "F", "Jp", "mat", "emitter")
_SHAPES = {"x": ((3,), np.float32), "v": ((3,), np.float32), "C": ((3, 3), np.float32), "F": ((3, 3), np.float32),
           "Jp": ((), np.float32), "mat": ((), np.int32), "emitter": ((), np.int32)}


class _PinnedPool:
    """Page-locked host buffers for asynchronous reads. A read leases one; the numpy arrays of that read keep
    the lease alive, and the buffer returns to the pool when the last of them is freed."""

    def __init__(self, lib):
        self.lib = lib
        self.free: list[tuple[int, int]] = []  # (address, bytes)
        self.closed = False

    def take(self, nbytes: int):
        for i, (addr, size) in enumerate(self.free):
            if size >= nbytes:
                return self.free.pop(i)
        p = C.c_void_p()
        _abi.check(self.lib.mpm_host_alloc(max(int(nbytes), 1 << 20) * 5 // 4, C.byref(p)))
        return p.value, max(int(nbytes), 1 << 20) * 5 // 4

    def give(self, block) -> None:
        if self.closed:
            self.lib.mpm_host_free(C.c_void_p(block[0]))
        else:
            self.free.append(block)

    def close(self) -> None:
        self.closed = True
        for addr, _ in self.free:
            self.lib.mpm_host_free(C.c_void_p(addr))
        self.free = []


class _Lease:
    def __init__(self, pool, block):
        self.pool, self.block = pool, block

    def __del__(self):
        try:
            self.pool.give(self.block)
        except Exception:
            pass


class PendingRead:
    """A read in flight (Gb300Solver.read_begin). wait() returns the arrays; they stay valid after later reads
    (each read has its own page-locked buffer, recycled when its arrays are freed)."""

    def __init__(self, solver, arrays):
        self._solver, self._arrays = solver, arrays

    def wait(self) -> dict[str, np.ndarray]:
        if self._solver is not None:
            self._solver._check(self._solver._lib.mpm_read_wait(self._solver._h))
            self._solver = None
        return self._arrays


def _f32(a, shape) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(shape))


def _i32(a, n) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, np.int32).reshape(n))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _device_index(device) -> int:
    if device is None:
        return 0
    s = str(device)
    if s.startswith("cuda"):
        return int(s.split(":")[1]) if ":" in s else 0
    raise ValueError(f"the gb300 backend runs on CUDA devices only, got device={device!r}")


class Gb300Solver(Solver):
    """MLS-MPM over one domain on one GB300 GPU."""

    def __init__(self, domain, materials: Sequence, gravity, particles_per_cell: int = 8, device: str | None = None,
                 frame_reads: bool = False):
        """frame_reads: get_particles reads the whole state in one copy and keeps it for a save_state that
        follows before the next change of the particles (the bake runner asks for both every frame,
        bake.py:195-201), so a frame costs one device-to-host read of 108 B per particle instead of 32 + 108."""
        super().__init__(domain, materials, gravity, particles_per_cell, device)
        self._lib = _abi.lib()
        self._h = C.c_void_p()
        self._frame_reads = bool(frame_reads)
        self._frame_state = None
        for m in self.materials:
            if m.model not in _abi.MODEL_IDS:
                raise NotImplementedError(f"material model {m.model!r} is not supported by the gb300 backend")
        d = domain_desc(domain)
        mats = (_abi.MpmMaterialDesc * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            mats[i] = _abi.MpmMaterialDesc(_abi.MODEL_IDS[m.model], m.youngs_modulus, m.poisson_ratio, m.density,
                                           m.yield_stress, m.friction_angle_deg, m.hardening, m.critical_compression,
                                           m.critical_stretch, m.max_hardening)
        g = (C.c_double * 3)(*self.gravity)
        self.device = device or "cuda:0"
        _abi.check(self._lib.mpm_create(C.byref(d), mats, len(self.materials), g, int(particles_per_cell),
                                        _device_index(self.device), C.byref(self._h)))
        self._n_colliders = 0

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.mpm_destroy(self._h)
            self._h = C.c_void_p()
        if hasattr(self, "_pool"):
            self._pool.close()  # buffers still leased by live arrays are freed when those arrays go
            del self._pool

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status: int) -> None:
        _abi.check(status, self._h)

    # -- particles ------------------------------------------------------------------------------------------
    def add_particles(self, positions, velocities, material_ids, emitter_ids) -> None:
        self._mutated()
        n = len(positions)
        if n == 0:
            return
        x, v = _f32(positions, (n, 3)), _f32(velocities, (n, 3))
        mat, em = _i32(material_ids, n), _i32(emitter_ids, n)
        self._check(self._lib.mpm_add_particles(self._h, n, _ptr(x), _ptr(v), _ptr(mat), _ptr(em)))

    @property
    def particle_count(self) -> int:
        n = C.c_int64()
        self._check(self._lib.mpm_particle_count(self._h, C.byref(n)))
        return n.value

    def _mutated(self) -> None:
        """The particles may have changed: a state kept by get_particles is stale."""
        self._frame_state = None

    def get_particles(self) -> ParticleData:
        if self._frame_reads:
            st = self._save_state()
            self._frame_state = st
            return ParticleData(st["x"], st["v"], st["mat"], st["emitter"])
        n = self.particle_count
        x, v = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        mat, em = np.empty(n, np.int32), np.empty(n, np.int32)
        self._check(self._lib.mpm_get_particles(self._h, _ptr(x), _ptr(v), _ptr(mat), _ptr(em)))
        return ParticleData(x, v, mat, em)

    def read_begin(self, keys=("x", "v", "mat", "emitter")) -> PendingRead:
        """Start reading the given state arrays (keys of save_state) without waiting: the copy runs beside the
        next advance; PendingRead.wait() returns them (mpm_read_begin / mpm_read_wait)."""
        n = self.particle_count
        if not hasattr(self, "_pool"):
            self._pool = _PinnedPool(self._lib)
        sizes = {k: n * int(np.prod(_SHAPES[k][0], dtype=np.int64)) * 4 for k in keys}
        total = sum(-(-b // 256) * 256 for b in sizes.values())
        block = self._pool.take(total)
        raw = (C.c_char * block[1]).from_address(block[0])
        raw._lease = _Lease(self._pool, block)
        arrays, ptrs, off = {}, {}, 0
        for k in keys:
            shape, dt = _SHAPES[k]
            arrays[k] = np.frombuffer(raw, dt, count=n * int(np.prod(shape, dtype=np.int64)), offset=off).reshape(
                (n, *shape))
            ptrs[k] = C.c_void_p(block[0] + off)
            off += -(-sizes[k] // 256) * 256
        del raw
        self._check(self._lib.mpm_read_begin(self._h, *(ptrs.get(k) for k in STATE_KEYS)))
        return PendingRead(self, arrays)

    def get_particles_async(self) -> PendingRead:
        """read_begin for the frame arrays; ParticleData(*wait()'s x, v, mat, emitter)."""
        return self.read_begin(("x", "v", "mat", "emitter"))

    def save_state(self) -> dict[str, np.ndarray]:
        if self._frame_state is not None:  # read by get_particles, nothing changed since
            st, self._frame_state = self._frame_state, None
            return st
        return self._save_state()

    def _save_state(self) -> dict[str, np.ndarray]:
        n = self.particle_count
        s = {"x": np.empty((n, 3), np.float32), "v": np.empty((n, 3), np.float32),
             "C": np.empty((n, 3, 3), np.float32), "F": np.empty((n, 3, 3), np.float32),
             "Jp": np.empty(n, np.float32), "mat": np.empty(n, np.int32), "emitter": np.empty(n, np.int32)}
        self._check(self._lib.mpm_save_state(self._h, *(_ptr(s[k]) for k in STATE_KEYS)))
        return s

    def load_state(self, state: dict[str, np.ndarray]) -> None:
        self._mutated()
        n = len(np.asarray(state["x"]).reshape(-1, 3))
        arrs = [_f32(state["x"], (n, 3)), _f32(state["v"], (n, 3)), _f32(state["C"], (n, 3, 3)),
                _f32(state["F"], (n, 3, 3)), _f32(state["Jp"], n), _i32(state["mat"], n), _i32(state["emitter"], n)]
        self._check(self._lib.mpm_load_state(self._h, n, *(_ptr(a) for a in arrs)))

    # -- colliders -------------------------------------------------------------------------------------------
    def set_colliders(self, colliders: Sequence[ColliderGeometry]) -> None:
        keep, descs = [], (_abi.MpmColliderDesc * max(1, len(colliders)))()
        for i, c in enumerate(colliders):
            verts = _f32(c.mesh.verts, (-1, 3))
            tris = np.ascontiguousarray(np.asarray(c.mesh.tris, np.int32).reshape(-1, 3))
            keep += [verts, tris]
            descs[i] = _abi.MpmColliderDesc(len(verts), len(tris), verts.ctypes.data, tris.ctypes.data,
                                            int(bool(c.closed)), float(c.friction))
        self._check(self._lib.mpm_set_colliders(self._h, len(colliders), descs))
        self._n_colliders = len(colliders)

    def set_collider_transforms(self, start: np.ndarray, end: np.ndarray) -> None:
        start = _f32(start, (-1, 4, 4))
        end = _f32(end, (-1, 4, 4))
        if len(start) != self._n_colliders or len(end) != self._n_colliders:
            raise ValueError(f"expected {self._n_colliders} collider transforms")
        self._check(self._lib.mpm_set_collider_transforms(self._h, len(start), _ptr(start), _ptr(end)))

    # -- stepping --------------------------------------------------------------------------------------------
    def advance(self, frame_dt: float) -> AdvanceStats:
        self._mutated()
        st = _abi.MpmAdvanceStats()
        self._check(self._lib.mpm_advance(self._h, float(frame_dt), C.byref(st)))
        return AdvanceStats(int(st.substeps), float(st.dt), int(st.removed))

    def substep(self, dt: float, s: float = 1.0, frame_dt: float = 1.0) -> None:
        """One substep with a given dt (fixed-dt runs and parity checks); asynchronous on the device."""
        self._mutated()
        self._check(self._lib.mpm_substep(self._h, float(dt), float(s), float(frame_dt)))

    def run_substeps(self, dt: float, count: int, frame_dt: float | None = None) -> None:
        """count substeps of a fixed dt in one call, as the substeps of one advance of frame_dt (default
        count * dt): no CFL choice, no removal of escaped particles."""
        self._mutated()
        fdt = float(frame_dt) if frame_dt is not None else float(dt) * int(count)
        self._check(self._lib.mpm_run_substeps(self._h, float(dt), int(count), fdt))

    def synchronize(self) -> None:
        self._check(self._lib.mpm_synchronize(self._h))

    # -- queries ---------------------------------------------------------------------------------------------
    def is_occupied(self, points: np.ndarray) -> np.ndarray:
        pts = _f32(points, (-1, 3))
        out = np.zeros(len(pts), np.uint8)
        if len(pts):
            self._check(self._lib.mpm_is_occupied(self._h, len(pts), _ptr(pts), _ptr(out)))
        return out.astype(bool)

    # -- measurement -----------------------------------------------------------------------------------------
    def set_option(self, option: int, value: int) -> None:
        self._check(self._lib.mpm_set_option(self._h, int(option), int(value)))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.mpm_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def kernel_times(self, reset: bool = False) -> dict[str, tuple[float, int]]:
        """Per-group (milliseconds, count) under OPT_KERNEL_TIMING 1."""
        return {k: v for k, v in self._times(reset).items() if k != "substep"}

    def substep_times(self, reset: bool = False) -> tuple[float, int]:
        """(milliseconds, substeps) of whole substeps under OPT_KERNEL_TIMING 2."""
        return self._times(reset)["substep"]

    def _times(self, reset: bool) -> dict[str, tuple[float, int]]:
        ms = (C.c_float * 5)()
        n = (C.c_int64 * 5)()
        self._check(self._lib.mpm_kernel_times(self._h, 5, ms, n, int(reset)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(_abi.KERNEL_SLOTS + ("substep",))}

    def grid_dims(self) -> tuple[int, int, int]:
        """Nodes per axis of the padded grid (grid shape + 6)."""
        dims = (C.c_int32 * 3)()
        self._check(self._lib.mpm_grid_dims(self._h, dims))
        return int(dims[0]), int(dims[1]), int(dims[2])

    def read_grid(self) -> np.ndarray:
        """(dims..., 4) float32: node velocity (momentum where the mass is 0) and mass after the last substep."""
        dims = self.grid_dims()
        out = np.zeros((dims[0], dims[1], dims[2], 4), np.float32)
        self._check(self._lib.mpm_read_grid(self._h, _ptr(out)))
        return out

    def read_collider_pose(self, c: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(M, M^-1, dM/dt) of collider c at the last substep, each 3x4."""
        M, Mi, dM = (np.zeros((3, 4), np.float32) for _ in range(3))
        self._check(self._lib.mpm_read_collider_pose(self._h, int(c), _ptr(M), _ptr(Mi), _ptr(dM)))
        return M, Mi, dM

    def launch_count(self) -> int:
        v = C.c_int64()
        self._check(self._lib.mpm_launch_count(self._h, C.byref(v)))
        return v.value

    def conservation(self) -> dict:
        """FP64 totals over the particles on the device: mass, momentum, centre of mass, kinetic energy."""
        out = np.zeros(9, np.float64)
        self._check(self._lib.mpm_conservation(self._h, out.ctypes.data_as(C.c_void_p)))
        m = out[0]
        return {"mass": m, "momentum": out[1:4].copy(), "com": out[4:7] / m if m > 0 else np.zeros(3),
                "ke": out[7], "non_finite": int(out[8])}

    def device_bytes(self) -> int:
        """Device memory this solver holds now."""
        n = C.c_int64()
        self._check(self._lib.mpm_device_bytes(self._h, C.byref(n)))
        return n.value

    def fp64_lanes(self) -> int:
        """SVD lanes whose FP32 sweeps did not converge (mpm_fp64_lanes)."""
        v = C.c_int64()
        self._check(self._lib.mpm_fp64_lanes(self._h, C.byref(v)))
        return v.value

    def fp64_redo_lanes(self) -> int:
        """Drucker-Prager / snow lanes G2P redid in FP64 (MPM_OPT_FP64_CLAMP) since the solver was created."""
        v = C.c_int64()
        self._check(self._lib.mpm_fp64_redo_lanes(self._h, C.byref(v)))
        return v.value

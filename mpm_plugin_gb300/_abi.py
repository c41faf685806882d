"""ctypes binding of ``include/mpm_gb300.h`` (the in-tree library ``_build/libmpm_gb300.so``).

There is no fallback: if the library is missing or cannot be loaded, importing the solver fails loudly.
Build it with ``python -m mpm_plugin_gb300.build`` (``__graft_entry__.build()`` does the same).
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmpm_gb300.so"

MPM_OK, MPM_ERR_VALUE, MPM_ERR_NOT_IMPLEMENTED, MPM_ERR_CUDA, MPM_ERR_ARGUMENT, MPM_ERR_MEMORY = range(6)
MODEL_IDS = {"elastic": 0, "von_mises": 1, "drucker_prager": 2, "snow": 3}
(OPT_USE_GRAPH, OPT_KERNEL_TIMING, OPT_SORT_INTERVAL, OPT_DETERMINISTIC, OPT_G2P_VARIANT, OPT_LIST_CTAS,
 OPT_P2G_GROUP, OPT_PDL, OPT_FP64_CLAMP, OPT_P2G_TILE, OPT_COOP, OPT_FUSED_P2G, OPT_BLOCK_SWEEP,
 OPT_PARTICLES_PER_THREAD, OPT_P2G_MERGE) = range(1, 16)
KERNEL_SLOTS = ("p2g", "grid_update", "g2p", "other")

# every symbol declared in include/mpm_gb300.h
EXPORTS = ("mpm_create", "mpm_destroy", "mpm_last_error", "mpm_add_particles", "mpm_set_colliders",
           "mpm_set_collider_transforms", "mpm_advance", "mpm_substep", "mpm_run_substeps", "mpm_particle_count", "mpm_get_particles",
           "mpm_is_occupied", "mpm_save_state", "mpm_load_state", "mpm_set_option", "mpm_get_stream",
           "mpm_synchronize", "mpm_kernel_times", "mpm_grid_dims", "mpm_read_grid", "mpm_read_collider_pose",
           "mpm_launch_count", "mpm_fp64_lanes", "mpm_fp64_redo_lanes", "mpm_is_occupied_noalloc", "mpm_volume_lattice", "mpm_read_begin", "mpm_read_wait", "mpm_host_alloc", "mpm_coop_barrier_selftest",
           "mpm_host_free", "mpm_conservation", "mpm_device_bytes", "mpm_batch_create", "mpm_batch_destroy",
           "mpm_batch_last_error", "mpm_batch_add", "mpm_batch_remove", "mpm_batch_size", "mpm_batch_advance",
           "mpm_batch_set_option", "mpm_batch_get_stream", "mpm_batch_launch_count", "mpm_surface_create",
           "mpm_surface_destroy", "mpm_surface_upload", "mpm_surface_last_error", "mpm_surface_build", "mpm_surface_read", "mpm_surface_read_field",
           "mpm_mc_table", "mpm_domain_grid_dims")


class MpmDomainDesc(C.Structure):
    _fields_ = [("min", C.c_double * 3), ("max", C.c_double * 3), ("resolution", C.c_int32),
                ("wall_lo", C.c_int32 * 3), ("wall_hi", C.c_int32 * 3), ("wall_friction", C.c_double)]


class MpmMaterialDesc(C.Structure):
    _fields_ = [("model", C.c_int32), ("youngs_modulus", C.c_double), ("poisson_ratio", C.c_double),
                ("density", C.c_double), ("yield_stress", C.c_double), ("friction_angle_deg", C.c_double),
                ("hardening", C.c_double), ("critical_compression", C.c_double), ("critical_stretch", C.c_double),
                ("max_hardening", C.c_double)]


class MpmColliderDesc(C.Structure):
    _fields_ = [("n_verts", C.c_int32), ("n_tris", C.c_int32), ("verts", C.c_void_p), ("tris", C.c_void_p),
                ("closed", C.c_int32), ("friction", C.c_double)]


class MpmAdvanceStats(C.Structure):
    _fields_ = [("substeps", C.c_int32), ("dt", C.c_double), ("removed", C.c_int32)]


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("MPM_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(f"the mpm_gb300 CUDA library is not built ({path}); run python -m mpm_plugin_gb300.build")
    L = C.CDLL(str(path))
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "mpm_create": [C.POINTER(MpmDomainDesc), C.POINTER(MpmMaterialDesc), I32, P, I32, I32, C.POINTER(P)],
        "mpm_destroy": [P],
        "mpm_add_particles": [P, I64, P, P, P, P],
        "mpm_set_colliders": [P, I32, P],
        "mpm_set_collider_transforms": [P, I32, P, P],
        "mpm_advance": [P, D, C.POINTER(MpmAdvanceStats)],
        "mpm_substep": [P, D, D, D],
        "mpm_run_substeps": [P, D, I32, D],
        "mpm_particle_count": [P, C.POINTER(I64)],
        "mpm_get_particles": [P, P, P, P, P],
        "mpm_is_occupied": [P, I64, P, P],
        "mpm_save_state": [P, P, P, P, P, P, P, P],
        "mpm_load_state": [P, I64, P, P, P, P, P, P, P],
        "mpm_set_option": [P, I32, I64],
        "mpm_get_stream": [P, C.POINTER(P)],
        "mpm_synchronize": [P],
        "mpm_kernel_times": [P, I32, P, P, I32],
        "mpm_grid_dims": [P, P],
        "mpm_domain_grid_dims": [C.POINTER(MpmDomainDesc), P],
        "mpm_read_grid": [P, P],
        "mpm_read_collider_pose": [P, I32, P, P, P],
        "mpm_launch_count": [P, C.POINTER(I64)],
        "mpm_fp64_lanes": [P, C.POINTER(I64)],
        "mpm_fp64_redo_lanes": [P, C.POINTER(I64)],
        "mpm_is_occupied_noalloc": [C.POINTER(MpmDomainDesc), I32, I64, P, I64, P, P, I32, P],
        "mpm_volume_lattice": [P, I64, P, I32, P, I32, P, I32, D, P, I64, I64, I32, P, I64, C.POINTER(I64)],
        "mpm_read_begin": [P, P, P, P, P, P, P, P],
        "mpm_read_wait": [P],
        "mpm_host_alloc": [I64, C.POINTER(P)],
        "mpm_host_free": [P],
        "mpm_conservation": [P, P],
        "mpm_device_bytes": [P, C.POINTER(I64)],
        "mpm_batch_create": [C.POINTER(P)],
        "mpm_batch_destroy": [P],
        "mpm_batch_add": [P, P],
        "mpm_batch_remove": [P, P],
        "mpm_batch_size": [P, C.POINTER(I32)],
        "mpm_batch_advance": [P, P, P],
        "mpm_batch_set_option": [P, I32, I64],
        "mpm_batch_get_stream": [P, C.POINTER(P)],
        "mpm_batch_launch_count": [P, C.POINTER(I64)],
        "mpm_coop_barrier_selftest": [P, I32, C.POINTER(I32)],
        "mpm_surface_create": [I32, C.POINTER(P)],
        "mpm_surface_destroy": [P],
        "mpm_surface_upload": [P, I64, P, P, P, P],
        "mpm_surface_build": [P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(I64),
                              C.POINTER(I64)],
        "mpm_surface_read": [P, P, P, P],
        "mpm_surface_read_field": [P, P, P],
        "mpm_mc_table": [P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.mpm_last_error.argtypes = [P]
    L.mpm_last_error.restype = C.c_char_p
    L.mpm_batch_last_error.argtypes = [P]
    L.mpm_batch_last_error.restype = C.c_char_p
    L.mpm_surface_last_error.argtypes = [P]
    L.mpm_surface_last_error.restype = C.c_char_p
    _lib = L
    return L


def check(status: int, handle=None, batch=None) -> None:
    """Map a status to the exception the reference raises in the same situation."""
    if status == MPM_OK:
        return
    err = lib().mpm_batch_last_error(batch) if batch is not None else lib().mpm_last_error(handle)
    msg = (err or b"").decode(errors="replace")
    if status == MPM_ERR_VALUE:
        raise ValueError(msg)
    if status == MPM_ERR_NOT_IMPLEMENTED:
        raise NotImplementedError(msg)
    if status == MPM_ERR_MEMORY:
        raise MemoryError(msg)
    if status == MPM_ERR_ARGUMENT:
        raise TypeError(msg)
    raise RuntimeError(f"CUDA error in the gb300 backend: {msg}")

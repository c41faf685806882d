"""The C-ABI library (CPU only: loading and symbols, no compute calls)."""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared() -> list[str]:
    text = (ROOT / "include" / "mpm_gb300.h").read_text()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(mpm_\w+)\(", text, flags=re.M)))


def test_header_lists_the_boundary():
    names = _declared()
    for required in ("mpm_create", "mpm_add_particles", "mpm_set_colliders", "mpm_set_collider_transforms",
                     "mpm_advance", "mpm_substep", "mpm_get_particles", "mpm_is_occupied", "mpm_save_state",
                     "mpm_load_state", "mpm_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from mpm_plugin_gb300 import _abi, build

    build.build()
    lib = _abi.lib()
    for name in _declared():
        assert hasattr(lib, name), name
    assert set(_abi.EXPORTS) == set(_declared())


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from mpm_plugin_gb300 import _abi

    monkeypatch.setattr(_abi, "_lib", None)
    monkeypatch.setenv("MPM_GB300_LIB", str(tmp_path / "nope.so"))
    with pytest.raises(ImportError, match="not built"):
        _abi.lib()


def test_status_mapping():
    from mpm_plugin_gb300 import _abi

    _abi.lib()
    with pytest.raises(ValueError):
        _abi.check(_abi.MPM_ERR_VALUE)
    with pytest.raises(NotImplementedError):
        _abi.check(_abi.MPM_ERR_NOT_IMPLEMENTED)
    with pytest.raises(RuntimeError):
        _abi.check(_abi.MPM_ERR_CUDA)
    _abi.check(_abi.MPM_OK)


def test_create_without_gpu_reports_cuda_error():
    """Host-side validation runs before any device call: an unknown model is NotImplementedError."""
    from mpm_plugin_gb300 import _abi

    L = _abi.lib()
    d = _abi.MpmDomainDesc()
    for a in range(3):
        d.max[a] = 1.0
        d.wall_lo[a] = d.wall_hi[a] = 1
    d.resolution = 8
    m = (_abi.MpmMaterialDesc * 1)()
    m[0].model = 7
    h = ctypes.c_void_p()
    g = (ctypes.c_double * 3)(0, 0, -9.81)
    assert L.mpm_create(ctypes.byref(d), m, 1, g, 8, 0, ctypes.byref(h)) == _abi.MPM_ERR_NOT_IMPLEMENTED
    assert b"not supported" in L.mpm_last_error(None)


@pytest.mark.parametrize("field,value,message", [
    ("resolution", 0, b"resolution"), ("resolution", -3, b"resolution"), ("max", 0.0, b"max must exceed min"),
    ("max", float("nan"), b"finite"), ("min", float("-inf"), b"finite")])
def test_bad_domain_descriptors_are_refused_before_the_device(field, value, message):
    """mpm_create and mpm_is_occupied_noalloc take a raw domain descriptor: a non-positive resolution,
    non-finite bounds or max <= min are value errors, found before any grid is derived or device touched."""
    from mpm_plugin_gb300 import _abi

    L = _abi.lib()
    d = _abi.MpmDomainDesc()
    for a in range(3):
        d.max[a] = 1.0
        d.wall_lo[a] = d.wall_hi[a] = 1
    d.resolution = 8
    if field == "resolution":
        d.resolution = value
    else:
        getattr(d, field)[2] = value
    m = (_abi.MpmMaterialDesc * 1)()
    h = ctypes.c_void_p()
    g = (ctypes.c_double * 3)(0, 0, -9.81)
    assert L.mpm_create(ctypes.byref(d), m, 1, g, 8, 0, ctypes.byref(h)) == _abi.MPM_ERR_VALUE
    assert message in L.mpm_last_error(None) and not h.value
    assert L.mpm_is_occupied_noalloc(ctypes.byref(d), 8, 0, None, 0, None, None, 0, None) == _abi.MPM_ERR_VALUE
    assert message in L.mpm_last_error(None)


def test_surfacer_entry_points_validate_before_the_device():
    """Surfacer calls with a null surfacer or null outputs fail with an argument error; without a GPU the
    creation fails with a CUDA error rather than crashing."""
    import ctypes as C

    from mpm_plugin_gb300 import _abi

    lib = _abi.lib()
    lo, hi = (C.c_float * 3)(), (C.c_float * 3)()
    assert lib.mpm_surface_upload(None, 10, None, None, lo, hi) == _abi.MPM_ERR_ARGUMENT
    nv, nt = C.c_int64(), C.c_int64()
    o, d = (C.c_float * 3)(), (C.c_int32 * 3)(4, 4, 4)
    assert lib.mpm_surface_build(None, o, d, 1.0, 1.0, 1.0, 1.0, 0.5, C.byref(nv), C.byref(nt)) == \
        _abi.MPM_ERR_ARGUMENT
    assert lib.mpm_surface_read(None, None, None, None) == _abi.MPM_ERR_ARGUMENT
    assert lib.mpm_surface_destroy(None) == _abi.MPM_OK
    assert lib.mpm_mc_table(None, None) == _abi.MPM_ERR_ARGUMENT
    s = C.c_void_p()
    import torch

    if not torch.cuda.is_available():
        assert lib.mpm_surface_create(0, C.byref(s)) == _abi.MPM_ERR_CUDA and not s.value
    flag = C.c_int32()
    assert lib.mpm_coop_barrier_selftest(None, 1, C.byref(flag)) == _abi.MPM_ERR_ARGUMENT

"""The occupancy query that allocates no device memory, against the regular one (GPU).

Some callers cannot allocate device memory when they query: a serving process whose device memory budget
was handed out at start-up, or a host application whose own allocator owns the device. For them
mpm_is_occupied_noalloc takes caller-owned device buffers and keeps its volume grid in a static 16 MiB
device array. This file is collected last, so a run that stops at the first failure has run every other
test before it.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
from scenes import add, box_particles, domain, preset

pytestmark = pytest.mark.gpu


def _domain_desc(d):
    from mpm_plugin_gb300 import _abi

    dd = _abi.MpmDomainDesc()
    for a, ax in enumerate("xyz"):
        dd.min[a], dd.max[a] = d.min[a], d.max[a]
        dd.wall_lo[a] = int(bool(d.walls[f"{ax}-"]))
        dd.wall_hi[a] = int(bool(d.walls[f"{ax}+"]))
    dd.resolution, dd.wall_friction = d.resolution, d.wall_friction
    return dd


def test_noalloc_occupancy_matches_regular_query_twice():
    import torch

    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.solver import Gb300Solver

    L = _abi.lib()
    d = domain(res=32)
    dd = _domain_desc(d)
    rng = np.random.default_rng(5)
    pts = rng.uniform(-0.05, 1.05, (4000, 3)).astype(np.float32)
    pts_d = torch.from_numpy(pts).cuda()
    out_d = torch.empty(len(pts), dtype=torch.uint8, device="cuda")
    # two calls in a row with different particles: the shared scratch must not carry the first call over
    sets = [box_particles((0.3, 0.3, 0.0), (0.7, 0.7, 0.3), d.dx, seed=1),
            box_particles((0.45, 0.45, 0.0), (0.55, 0.55, 0.1), d.dx, seed=2)]
    for x in sets:
        s = Gb300Solver(d, [preset("jelly")], (0.0, 0.0, -9.81), 8, device="cuda:0")
        add(s, x)
        expected = s.is_occupied(pts)
        x_d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        out_d.fill_(7)
        torch.cuda.synchronize()
        status = L.mpm_is_occupied_noalloc(C.byref(dd), 8, len(x), C.c_void_p(x_d.data_ptr()), len(pts),
                                           C.c_void_p(pts_d.data_ptr()), C.c_void_p(out_d.data_ptr()), 0, None)
        assert status == _abi.MPM_OK, L.mpm_last_error(None)
        torch.cuda.synchronize()
        got = out_d.cpu().numpy()
        assert set(np.unique(got)) <= {0, 1}
        np.testing.assert_array_equal(got.astype(bool), expected)
        assert expected.any() and not expected.all()
        s.close()


def test_noalloc_on_a_caller_stream_and_with_no_particles():
    """On a stream the caller owns (not the legacy default one): with no particles nothing is occupied, and a
    call with particles right after it on the same stream answers as the regular query does."""
    import torch

    from mpm_plugin_gb300 import _abi
    from mpm_plugin_gb300.solver import Gb300Solver

    L = _abi.lib()
    d = domain(res=24)
    dd = _domain_desc(d)
    pts = np.random.default_rng(9).uniform(0.0, 1.0, (3000, 3)).astype(np.float32)
    x = box_particles((0.2, 0.2, 0.0), (0.6, 0.5, 0.4), d.dx, seed=3)
    s = Gb300Solver(d, [preset("jelly")], (0.0, 0.0, -9.81), 8, device="cuda:0")
    add(s, x)
    expected = s.is_occupied(pts)
    s.close()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        pts_d = torch.from_numpy(pts).cuda()
        x_d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        out_d = torch.full((len(pts),), 7, dtype=torch.uint8, device="cuda")
    empty = L.mpm_is_occupied_noalloc(C.byref(dd), 8, 0, None, len(pts), C.c_void_p(pts_d.data_ptr()),
                                      C.c_void_p(out_d.data_ptr()), 0, C.c_void_p(stream.cuda_stream))
    assert empty == _abi.MPM_OK, L.mpm_last_error(None)
    stream.synchronize()
    assert not out_d.cpu().numpy().any()
    full = L.mpm_is_occupied_noalloc(C.byref(dd), 8, len(x), C.c_void_p(x_d.data_ptr()), len(pts),
                                     C.c_void_p(pts_d.data_ptr()), C.c_void_p(out_d.data_ptr()), 0,
                                     C.c_void_p(stream.cuda_stream))
    assert full == _abi.MPM_OK, L.mpm_last_error(None)
    stream.synchronize()
    np.testing.assert_array_equal(out_d.cpu().numpy().astype(bool), expected)


def test_noalloc_refuses_a_domain_beyond_its_scratch():
    from mpm_plugin_gb300 import _abi

    L = _abi.lib()
    dd = _domain_desc(domain(res=256))
    x = np.zeros((1, 3), np.float32)
    out = np.zeros(1, np.uint8)
    status = L.mpm_is_occupied_noalloc(C.byref(dd), 8, 0, None, 1, C.c_void_p(x.ctypes.data),
                                       C.c_void_p(out.ctypes.data), 0, None)
    assert status == _abi.MPM_ERR_VALUE
    assert b"static scratch" in L.mpm_last_error(None)


@pytest.mark.parametrize("field,value,message", [
    ("resolution", 0, b"resolution"), ("max0", 0.0, b"max must exceed min"), ("min1", float("nan"), b"finite")])
def test_noalloc_refuses_bad_domains_and_devices(field, value, message):
    """A raw descriptor is checked before any grid is derived from it, and a device index beyond the device
    count is refused before any device is made current."""
    from mpm_plugin_gb300 import _abi

    L = _abi.lib()
    dd = _domain_desc(domain(res=16))
    if field == "resolution":
        dd.resolution = value
    elif field == "max0":
        dd.max[0] = value
    else:
        dd.min[1] = value
    x = np.zeros((1, 3), np.float32)
    out = np.zeros(1, np.uint8)
    status = L.mpm_is_occupied_noalloc(C.byref(dd), 8, 0, None, 1, C.c_void_p(x.ctypes.data),
                                       C.c_void_p(out.ctypes.data), 0, None)
    assert status == _abi.MPM_ERR_VALUE and message in L.mpm_last_error(None)
    good = _domain_desc(domain(res=16))
    status = L.mpm_is_occupied_noalloc(C.byref(good), 8, 0, None, 1, C.c_void_p(x.ctypes.data),
                                       C.c_void_p(out.ctypes.data), 4096, None)
    assert status == _abi.MPM_ERR_ARGUMENT and b"device index" in L.mpm_last_error(None)

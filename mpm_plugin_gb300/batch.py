"""Gb300Batch: many independent scenes (Gb300Solver instances on one GPU) advanced together.

The reference advances one scene per ``Solver.advance`` call (mpm_core/solver.py:67-68). A batch keeps that
per-scene contract (each scene's own CFL time step, materials, colliders, particle order, statistics) and
runs every kernel of a substep once for all of its scenes, so many small scenes fill the GPU together and
pay the launch and synchronisation costs of one.
"""

from __future__ import annotations

import ctypes as C
from collections.abc import Sequence

import numpy as np

from mpm_plugin_gb300 import _abi
from mpm_plugin_gb300.interface import AdvanceStats


class Gb300Batch:
    def __init__(self, solvers: Sequence = ()):
        self._lib = _abi.lib()
        self._b = C.c_void_p()
        self._check(self._lib.mpm_batch_create(C.byref(self._b)))
        self._scenes: list = []
        for s in solvers:
            self.add(s)

    def _check(self, status: int) -> None:
        _abi.check(status, batch=self._b)

    def close(self) -> None:
        if getattr(self, "_b", None) and self._b.value:
            self._lib.mpm_batch_destroy(self._b)
            self._b = C.c_void_p()
            self._scenes = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self) -> int:
        return len(self._scenes)

    @property
    def scenes(self) -> list:
        return list(self._scenes)

    def add(self, solver) -> None:
        """The solver joins the batch; it stays usable on its own (its work then runs on the batch's stream)."""
        self._check(self._lib.mpm_batch_add(self._b, solver._h))
        self._scenes.append(solver)

    def remove(self, solver) -> None:
        self._check(self._lib.mpm_batch_remove(self._b, solver._h))
        self._scenes.remove(solver)

    def advance(self, frame_dt) -> list[AdvanceStats]:
        """One frame of every scene; frame_dt is one value for all or one per scene (in the order added)."""
        self._scenes = [s for s in self._scenes if s._h.value]  # a closed solver has left the batch
        n = len(self._scenes)
        if n == 0:
            return []
        fdt = np.broadcast_to(np.asarray(frame_dt, np.float64), (n,)).copy()
        for s in self._scenes:
            s._mutated()
        stats = (_abi.MpmAdvanceStats * n)()
        self._check(self._lib.mpm_batch_advance(self._b, fdt.ctypes.data_as(C.c_void_p), stats))
        return [AdvanceStats(int(st.substeps), float(st.dt), int(st.removed)) for st in stats]

    def set_option(self, option: int, value: int) -> None:
        self._check(self._lib.mpm_batch_set_option(self._b, int(option), int(value)))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.mpm_batch_get_stream(self._b, C.byref(s)))
        return s.value or 0

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self._lib.mpm_batch_launch_count(self._b, C.byref(n)))
        return n.value

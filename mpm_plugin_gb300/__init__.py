"""GB300-native (sm_103a) MLS-MPM substep backend for the reference's ``mpm_core`` solver interface.

``Gb300Solver`` implements ``mpm_core.solver.Solver`` over hand-written CUDA kernels reached through the
C-ABI in ``include/mpm_gb300.h``. Importing this package registers it as backend ``"gb300"`` with
``mpm_core.backends`` when the reference package is importable, so the bake runner selects it with
``--backend gb300`` (see ``python -m mpm_plugin_gb300.bake``).
"""

from mpm_plugin_gb300.interface import HAVE_MPM_CORE

BACKEND_NAME = "gb300"


def create(**kwargs):
    """Factory with the signature ``create_solver`` passes (mpm_core/backends/__init__.py:25-28)."""
    from mpm_plugin_gb300.solver import Gb300Solver

    return Gb300Solver(**kwargs)


def register() -> bool:
    """Register ``"gb300"`` with ``mpm_core.backends``; False when the reference package is absent."""
    if not HAVE_MPM_CORE:
        return False
    from mpm_core.backends import register_backend

    register_backend(BACKEND_NAME, create)
    return True


register()

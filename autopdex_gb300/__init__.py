"""GB300-native solve backend for AutoPDEx.

Select it with ``static_settings['solver backend'] = 'gb300'`` and call
``autopdex_gb300.solver.solver(dofs, settings, static_settings)`` in place of
``autopdex.solver.solver``.  Element assembly, the node-block CSR scatter with Dirichlet
elimination, the Krylov solves and the Newton loop run as sm_103a CUDA kernels in
``libautopdex_gb300.so`` (C ABI: include/autopdex_gb300.h).
"""
from . import geometry, mesher, models, seeder, spaces, utility  # noqa: F401

__all__ = ["geometry", "mesher", "models", "seeder", "spaces", "utility", "solver", "assembler"]


def __getattr__(name):
    # solver/assembler import torch and load the native library lazily
    if name in ("solver", "assembler"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)

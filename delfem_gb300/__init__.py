"""delfem_gb300 -- GB300 (sm_103a) implementation of DelFEM's FE assembly +
block ILU(0)-preconditioned CG hot path behind a C ABI (include/dfg.h).

The compute path is libdfg.so (CUDA kernels + C++ host code, built in-tree by
``delfem_gb300.build``); this package only binds it.  There is no CPU
fallback: a missing or unloadable library raises.
"""
from . import capi, meshgen  # noqa: F401
from .capi import DfgError, lib  # noqa: F401

__all__ = ["capi", "meshgen", "lib", "DfgError", "linsys", "solver"]


def __getattr__(name):
    if name in ("linsys", "solver"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)

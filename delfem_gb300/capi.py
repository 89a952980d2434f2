"""ctypes binding of libdfg's C ABI (include/dfg.h).

The library is loaded from the package directory (built in-tree by
``delfem_gb300.build``).  There is no fallback: if the shared library is
missing or cannot be loaded, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdfg.so")
HEADER = os.path.join(HERE, "..", "include", "dfg.h")

DFG_OK = 0
DFG_NOT_CONVERGED = 1
DFG_SINGULAR_PIVOT = 2
DFG_NAN_DETECTED = 3
DFG_OOM_REJECTED = 4
DFG_TIMEOUT = 5
DFG_INVALID_ARGUMENT = 6
DFG_CUDA_ERROR = 7
DFG_NOT_READY = 8
DFG_PREC_FP64 = 0
DFG_PREC_MIXED = 1
DFG_PREC_FP32_FACTOR = 2
MODES = {"fp64": DFG_PREC_FP64, "mixed": DFG_PREC_MIXED, "fp32f": DFG_PREC_FP32_FACTOR}
STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "SINGULAR_PIVOT", 3: "NAN_DETECTED", 4: "OOM_REJECTED",
                5: "TIMEOUT", 6: "INVALID_ARGUMENT", 7: "CUDA_ERROR", 8: "NOT_READY"}

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_U = ctypes.c_uint
_LL = ctypes.c_longlong
_PI = ctypes.POINTER(ctypes.c_int)
_PD = ctypes.POINTER(ctypes.c_double)
_PU = ctypes.POINTER(ctypes.c_uint)

# name -> (restype, argtypes)
SIGNATURES = {
    "dfg_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "dfg_ctx_destroy": (_I, [_P]),
    "dfg_last_error": (ctypes.c_char_p, [_P]),
    "dfg_version": (ctypes.c_char_p, []),
    "dfg_ctx_synchronize": (_I, [_P]),
    "dfg_ctx_kernel_launches": (_LL, [_P]),
    "dfg_system_create": (_I, [_P, _I, _I, _P, _P, ctypes.POINTER(_P)]),
    "dfg_system_create_from_elements": (_I, [_P, _I, _I, _I, _I, _P, ctypes.POINTER(_P)]),
    "dfg_system_destroy": (_I, [_P]),
    "dfg_system_info": (_I, [_P, _PI, _PI, ctypes.POINTER(_LL)]),
    "dfg_system_get_pattern": (_I, [_P, _P, _P]),
    "dfg_system_set_mesh": (_I, [_P, _I, _P, _I, _I, _P]),
    "dfg_system_set_coef": (_I, [_P, _P]),
    "dfg_system_set_field": (_I, [_P, _P, _P]),
    "dfg_system_update_field": (_I, [_P, _I]),
    "dfg_system_get_field": (_I, [_P, _P, _P]),
    "dfg_mesh_read_gid": (_I, [ctypes.c_char_p, _PI, _PI, _PI, _PI, _P, _P]),
    "dfg_set_bcflags": (_I, [_P, _P]),
    "dfg_initialize_marge": (_I, [_P]),
    "dfg_assemble_poisson": (_I, [_P, _D, _D]),
    "dfg_assemble_diffusion": (_I, [_P, _D, _D, _D, _D, _D]),
    "dfg_assemble_solid2d": (_I, [_P, _D, _D, _D, _D, _D]),
    "dfg_assemble_solid3d": (_I, [_P, _D, _D, _D, _D, _D, _D]),
    "dfg_add_residual": (_I, [_P, _P]),
    "dfg_system_set_load": (_I, [_P, _P]),
    "dfg_finalize_marge": (_I, [_P, _PD]),
    "dfg_get_matrix": (_I, [_P, _P, _P]),
    "dfg_set_matrix": (_I, [_P, _P, _P]),
    "dfg_get_vector": (_I, [_P, _I, _P]),
    "dfg_set_vector": (_I, [_P, _I, _P]),
    "dfg_get_tmp_vector_size": (_I, [_P, _PU]),
    "dfg_resize_tmp_vec": (_I, [_P, _U]),
    "dfg_dot": (_I, [_P, _I, _I, _PD]),
    "dfg_copy": (_I, [_P, _I, _I]),
    "dfg_scal": (_I, [_P, _D, _I]),
    "dfg_axpy": (_I, [_P, _D, _I, _I]),
    "dfg_matvec": (_I, [_P, _D, _I, _D, _I]),
    "dfg_precond_create": (_I, [_P, ctypes.POINTER(_P)]),
    "dfg_precond_destroy": (_I, [_P]),
    "dfg_precond_set_fill_level": (_I, [_P, _I]),
    "dfg_precond_set_linear_system": (_I, [_P, _P]),
    "dfg_precond_set_value": (_I, [_P, _P]),
    "dfg_precond_solve": (_I, [_P, _P, _I]),
    "dfg_precond_get_factor": (_I, [_P, _P, _P]),
    "dfg_precond_get_pattern": (_I, [_P, _P, _P, _P]),
    "dfg_precond_set_sweep_mode": (_I, [_P, _I]),
    "dfg_precond_get_sweep_mode": (_I, [_P, _PI, _PI]),
    "dfg_precond_get_sweep_timing": (_I, [_P, _P]),
    "dfg_precond_get_solo_timing": (_I, [_P, _P]),
    "dfg_solve_pcg": (_I, [_P, _P, _PD, _PU]),
    "dfg_solve_pcg_mixed": (_I, [_P, _P, _PD, _PU, _PU]),
    "dfg_solve_pcg_ex": (_I, [_P, _P, _I, _I, _PD, _PU, _PU]),
    "dfg_solve_pbicgstab": (_I, [_P, _P, _I, _PD, _PU]),
    "dfg_true_residual": (_I, [_P, _P, _PD]),
    "dfg_ctx_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "dfg_profile_kernels": (_I, [_P, _P, _I, _I, _P, _P]),
    "dfg_dot_noalloc": (_I, [_P, _P, _LL, _PD, _P]),
    "dfg_server_create": (_I, [_P, _P, ctypes.POINTER(_P)]),
    "dfg_server_submit": (_I, [_P, _P, ctypes.POINTER(_LL)]),
    "dfg_server_wait": (_I, [_P, _LL, _P]),
    "dfg_server_error_text": (_I, [_P, _LL, ctypes.c_char_p, _I]),
    "dfg_server_drain": (_I, [_P]),
    "dfg_server_stats": (_I, [_P, _P]),
    "dfg_server_destroy": (_I, [_P]),
    "dfg_server_profile": (_I, [_P, _P]),
    "dfg_selftest_wait_timeout": (_I, [_P, _PI]),
}


class ServerConfig(ctypes.Structure):
    """dfg_server_config"""
    _fields_ = [("mode", _I), ("tol", _D), ("maxit", _I), ("budget_bytes", _LL), ("max_inflight", _I),
                ("chunk_iters", _I), ("host_threads", _I), ("profile_every", _I), ("size_groups", _I),
                ("sweeps", _I)]


class Request(ctypes.Structure):
    """dfg_request"""
    _fields_ = [("kind", _I), ("nnode", _I), ("nelem", _I), ("coords", _P), ("conn", _P), ("coef", _P),
                ("params", _P), ("nparams", _I), ("bcflag", _P), ("load", _P), ("x_out", _P)]


class Result(ctypes.Structure):
    """dfg_result"""
    _fields_ = [("id", _LL), ("status", _I), ("iterations", _I), ("conv", _D), ("rel_true", _D),
                ("t_submit", _D), ("t_admit", _D), ("t_done", _D), ("device_bytes", _LL)]


class ServerCounters(ctypes.Structure):
    """dfg_server_counters"""
    _fields_ = [("submitted", _LL), ("finished", _LL), ("replays", _LL), ("kernel_launches", _LL),
                ("graph_builds", _LL), ("peak_inflight", _LL), ("budget_bytes", _LL), ("peak_bytes", _LL),
                ("h2d_bytes", _LL), ("d2h_bytes", _LL), ("busy_seconds", _D), ("now_seconds", _D),
                ("backlog_seconds", _D), ("queued_seconds", _D), ("full_seconds", _D),
                ("inflight_seconds", _D), ("symbolic_seconds", _D), ("admit_seconds", _D)]


SERVER_NKERNELS = 24
SERVER_KERNEL_NAMES = ["rz_beta", "update_p", "spmv_pap", "update_rx", "check_true", "replace"] + [
    f"sweep_{d}_b{c // 3 + 1}_e{(4, 8, 16)[c % 3]}" for c in range(9) for d in ("fwd", "bwd")]


class ServerProfile(ctypes.Structure):
    """dfg_server_profile_t"""
    _fields_ = [("ms", _D * SERVER_NKERNELS), ("bytes", _D * SERVER_NKERNELS), ("n", _LL * SERVER_NKERNELS)]


DFG_DOT_NOALLOC_MAX_LEN = 33554432

_lib = None


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dfg_[a-z0-9_]+)\s*\(", txt)))


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libdfg is not built ({LIB_PATH} missing); run delfem_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class DfgError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(ctx, status: int, where: str) -> int:
    if status != DFG_OK:
        msg = lib().dfg_last_error(ctx).decode(errors="replace") if ctx else ""
        raise DfgError(status, where, msg)
    return status

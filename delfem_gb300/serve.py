"""Serving: many FE solves resident on one device, iterated together.

``Server`` mirrors the C ABI's ``dfg_server_*`` (include/dfg.h): requests are
``meshgen.Problem`` instances; each is admitted when its device bytes fit the
server's budget and a slot is free, assembled, factorised (ILU(0)) and solved
by PCG in batched launches with every other solve in flight.  The reference
has no serving layer; each solve follows its AddLinSys_* -> FinalizeMarge ->
CPreconditioner_ILU -> Solve_PCG path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from . import meshgen as mg
from .capi import check, lib

MODES = {"fp64": capi.DFG_PREC_FP64, "fp32f": capi.DFG_PREC_FP32_FACTOR, "mixed": capi.DFG_PREC_MIXED}


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Server:
    def __init__(self, ctx, mode: str = "fp32f", tol: float = 1e-8, maxit: int = 20000, budget_bytes: int = 0,
                 max_inflight: int = 0, chunk_iters: int = 8, host_threads: int = 0, profile_every: int = 0,
                 size_groups: int = 0, sweeps: int = 0):
        self.ctx = ctx
        cfg = capi.ServerConfig(MODES[mode], tol, maxit, budget_bytes, max_inflight, chunk_iters, host_threads,
                                profile_every, size_groups, sweeps)
        h = ctypes.c_void_p()
        check(ctx.h, lib().dfg_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(h)), "dfg_server_create")
        self.h = h
        if hasattr(ctx, "adopt"):
            ctx.adopt(self)
        self.mode = mode
        self._out: dict[int, np.ndarray] = {}

    def submit(self, p: mg.Problem, x_out: np.ndarray | None = None) -> int:
        """Queues one solve; the solution lands in ``x_out`` (allocated here
        if not given) before the request completes."""
        coords = np.ascontiguousarray(p.coords, dtype=np.float64)
        conn = np.ascontiguousarray(p.conn, dtype=np.int32)
        coef = None if p.coef is None else np.ascontiguousarray(p.coef, dtype=np.float64)
        params = np.ascontiguousarray(p.params, dtype=np.float64)
        bc = np.ascontiguousarray(p.bcflag, dtype=np.int32)
        load = None if p.load is None else np.ascontiguousarray(p.load, dtype=np.float64)
        if x_out is None:
            x_out = np.zeros(p.nnode * p.b)
        assert x_out.dtype == np.float64 and x_out.flags.c_contiguous and x_out.size == p.nnode * p.b
        req = capi.Request(p.kind, p.nnode, p.nelem, _ptr(coords), _ptr(conn), _ptr(coef), _ptr(params),
                           min(len(params), 8), _ptr(bc), _ptr(load), _ptr(x_out))
        rid = ctypes.c_longlong()
        check(self.ctx.h, lib().dfg_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)), "dfg_server_submit")
        self._out[rid.value] = x_out
        return rid.value

    def wait(self, rid: int) -> dict:
        r = capi.Result()
        check(self.ctx.h, lib().dfg_server_wait(self.h, rid, ctypes.byref(r)), "dfg_server_wait")
        out = {f: getattr(r, f) for f, _ in capi.Result._fields_}
        out["x"] = self._out[rid]
        if r.status != capi.DFG_OK:
            buf = ctypes.create_string_buffer(512)
            lib().dfg_server_error_text(self.h, rid, buf, 512)
            out["error"] = buf.value.decode(errors="replace")
        return out

    def release(self, rid: int) -> None:
        """Drops this side's reference to a finished request's solution buffer."""
        self._out.pop(rid, None)

    def drain(self) -> int:
        return lib().dfg_server_drain(self.h)

    def stats(self) -> dict:
        c = capi.ServerCounters()
        check(self.ctx.h, lib().dfg_server_stats(self.h, ctypes.byref(c)), "dfg_server_stats")
        return {f: getattr(c, f) for f, _ in capi.ServerCounters._fields_}

    def profile(self) -> dict:
        """Per batched kernel: launches profiled, mean ms per launch, mean
        algorithmic bytes per launch and the GB/s they imply."""
        pr = capi.ServerProfile()
        check(self.ctx.h, lib().dfg_server_profile(self.h, ctypes.byref(pr)), "dfg_server_profile")
        out = {}
        for k, name in enumerate(capi.SERVER_KERNEL_NAMES):
            n = pr.n[k]
            if n:
                ms = pr.ms[k] / n
                by = pr.bytes[k] / n
                out[name] = {"n": n, "ms": ms, "bytes": by, "gbs": (by / (ms * 1e-3) / 1e9) if ms > 0 and by > 0 else None}
        return out

    _close_order = 0

    def close(self) -> None:
        if getattr(self, "h", None):
            if self.ctx.h:  # after its context the handle is only dropped
                lib().dfg_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

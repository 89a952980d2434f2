"""dfg_dot_noalloc (the allocation-free dot product) against dfg_dot, through
the C ABI.

The vectors live in device memory the test owns (torch tensors, plumbing
only); the entry point itself allocates nothing.  The two dot products sum in
different block partitions, so they agree to rounding: the bar is
|a - b| <= 1e-12 * sum_i |x_i y_i| (the summation error scale).  Two calls in
a row must each meet it and give the same bits.  This file runs last (file
name), and it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(ctx, m):
    """A 1x1-block system of m rows with a chain pattern: slots 0 and 1 hold x, y."""
    from delfem_gb300 import linsys as L
    i = np.arange(m, dtype=np.int64)
    nb = np.stack([i - 1, i + 1], axis=1)
    keep = (nb >= 0) & (nb < m)
    rowptr = np.concatenate([[0], np.cumsum(keep.sum(axis=1))]).astype(np.int32)
    colind = nb[keep].astype(np.int32)
    return L.LinearSystemField(ctx, m, 1, rowptr=rowptr, colind=colind)


def _noalloc(xd, yd, m, stream=None):
    from delfem_gb300 import capi
    out = ctypes.c_double(np.nan)
    st = capi.lib().dfg_dot_noalloc(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()), m,
                                    ctypes.byref(out), stream)
    return st, out.value


@pytest.mark.parametrize("m", [1, 4095, 4097, 100_003])
def test_noalloc_matches_dfg_dot(gpu_ctx, m):
    import torch
    from delfem_gb300 import capi
    rng = np.random.default_rng(m)
    x = rng.standard_normal(m)
    y = rng.standard_normal(m) * np.exp(rng.standard_normal(m))
    ls = _system(gpu_ctx, m)
    ls.ReSizeTmpVecSolver(2)
    ls.SetVector(0, x)
    ls.SetVector(1, y)
    ref = ls.DOT(0, 1)
    torch.cuda.synchronize()
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y).cuda()
    torch.cuda.synchronize()
    bound = 1e-12 * float(np.abs(x * y).sum())
    st1, d1 = _noalloc(xd, yd, m)
    st2, d2 = _noalloc(xd, yd, m)
    assert st1 == capi.DFG_OK and st2 == capi.DFG_OK
    assert abs(d1 - ref) <= bound, (d1, ref, bound)
    assert abs(d2 - ref) <= bound, (d2, ref, bound)
    assert np.float64(d1).view(np.uint64) == np.float64(d2).view(np.uint64)
    ls.close()


def test_noalloc_at_the_maximum_length_and_beyond(gpu_ctx):
    import torch
    from delfem_gb300 import capi
    m = capi.DFG_DOT_NOALLOC_MAX_LEN
    g = torch.Generator(device="cuda").manual_seed(7)
    xd = torch.rand(m, dtype=torch.float64, device="cuda", generator=g) - 0.5
    yd = torch.rand(m, dtype=torch.float64, device="cuda", generator=g) - 0.5
    torch.cuda.synchronize()
    # m at the limit: compared with dfg_dot over the same values
    ls = _system(gpu_ctx, m)
    ls.ReSizeTmpVecSolver(2)
    x = xd.cpu().numpy()
    y = yd.cpu().numpy()
    ls.SetVector(0, x)
    ls.SetVector(1, y)
    ref = ls.DOT(0, 1)
    bound = 1e-12 * float(np.abs(x * y).sum())
    for _ in range(2):
        st, d = _noalloc(xd, yd, m)
        assert st == capi.DFG_OK and abs(d - ref) <= bound, (d, ref, bound)
    ls.close()
    # one element more is rejected before any device work, with a reason
    st, _ = _noalloc(xd, yd, m + 1)
    assert st == capi.DFG_INVALID_ARGUMENT
    assert b"exceeds the maximum" in capi.lib().dfg_last_error(None)


def test_noalloc_empty_and_bad_arguments(gpu_ctx):
    from delfem_gb300 import capi
    L = capi.lib()
    out = ctypes.c_double(np.nan)
    assert L.dfg_dot_noalloc(None, None, 0, ctypes.byref(out), None) == capi.DFG_OK and out.value == 0.0
    assert L.dfg_dot_noalloc(None, None, -1, ctypes.byref(out), None) == capi.DFG_INVALID_ARGUMENT
    assert L.dfg_dot_noalloc(None, None, 5, ctypes.byref(out), None) == capi.DFG_INVALID_ARGUMENT

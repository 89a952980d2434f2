"""Device memory is returned: repeated create / solve / destroy cycles of
every handle kind (systems built on the device, ILU(0) and ILU(1)
preconditioners, PCG in all precision modes, BiCGSTAB, a server) leave the
device's free memory where it was."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _free_bytes():
    """Device-wide free memory (cudaMemGetInfo, through torch when present)."""
    try:
        import torch
        torch.cuda.synchronize()
        return torch.cuda.mem_get_info()[0]
    except ImportError:
        import ctypes.util
        name = ctypes.util.find_library("cudart")
        if not name:
            pytest.skip("no way to read the device's free memory")
        rt = ctypes.CDLL(name)
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
        return free.value


def _cycle(ctx):
    from delfem_gb300 import linsys as L
    from delfem_gb300 import meshgen as mg
    from delfem_gb300.serve import Server
    from delfem_gb300.solver import FESolve
    p = mg.solid2d_cantilever(60, 24, seed=61, coef_sigma=0.5)
    for lev in (0, 1):
        s = FESolve(ctx, p, fill_level=lev)
        for mode in ("fp64", "fp32f", "mixed"):
            assert s.run(mode, target_true=True)["converged"]
        s.assemble()
        s.factor()
        ok, _, _ = L.Solve_PBiCGSTAB(1e-8, 2000, s.ls, s.prec)
        assert ok
        s.close()
    probs = [it.problem() for it in mg.serve_stream_2d(nreq=3, seed=62, nmin=500, nmax=2000)]
    with Server(ctx, mode="fp32f", budget_bytes=128 << 20) as S:
        ids = [S.submit(q) for q in probs]
        assert all(S.wait(i)["status"] == 0 for i in ids)
    ctx.synchronize()


def test_cycles_return_device_memory(gpu_ctx):
    _cycle(gpu_ctx)  # first cycle: one-time allocations (scratch, module loading)
    before = _free_bytes()
    for _ in range(3):
        _cycle(gpu_ctx)
    after = _free_bytes()
    assert before - after <= 8 << 20, (before, after)

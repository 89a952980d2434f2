"""The multi-rank bench logic on CPU: two `gloo` ranks on 127.0.0.1.

The GPU runs use NCCL with one rank per GPU; the reduction helpers and the
reference arm's rank-0-only rule are backend-independent and are checked here
without a GPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import torch.distributed as dist
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    wall = 2.0 + rank          # rank 1 is the slower one
    out = dict(rank=rank,
               env=bench.dist_env(),
               maxwall=bench.max_over_ranks(wall, world),
               rate=bench.whole_job_rate(100, wall, world))

    class Args:
        config, steps, warmup, ref_sample_every, serve_requests, cpu_sample_iters = "serve2d", 1, 3, 1, 4, 1
    if rank != 0:
        out["ref_line"] = bench.run_reference(Args, rank, world)   # rank > 0 does no work
    dist.barrier()
    dist.destroy_process_group()
    q.put(out)


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = sorted((q.get(timeout=120) for _ in procs), key=lambda o: o["rank"])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for o in outs:
        assert o["env"] == (o["rank"], 2, o["rank"])
        assert o["maxwall"] == 3.0                      # max over ranks
        assert o["rate"] == pytest.approx(200 / 3.0)    # both ranks' units over the slowest time
    assert outs[1]["ref_line"] is None

"""Multi-GPU host logic on CPU: one DBS instance per rank (seed 1 + rank),
whole-job work summed over ranks and time taken as the max over ranks, with
two gloo ranks on 127.0.0.1."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys

    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r "ran" an instance with seed 1 + r: different work and time per rank
    r = {"wall": 1.0 + rank, "dev_s": 0.5 + 2 * rank, "evals": 10 * (rank + 1), "accepts": rank + 3,
         "launched": 100 + rank}
    res = bench.reduce_form(r, dist, device="cpu")
    out[rank] = res
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank in range(2):
        wall, dev, evals, accepts, launched = out[rank]
        assert wall == 2.0 and dev == 2.5          # max over ranks
        assert evals == 30 and accepts == 7 and launched == 201  # sums over ranks

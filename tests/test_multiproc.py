"""Multi-rank logic on CPU (gloo, world size 2).

The Fock build shards by quartets: each rank builds partial J/K from its share
of the quartets and one all-reduce (SUM) of J and K completes them (the
partition hook is sf_set_partition on the GPU).  Here every rank evaluates its
share with the oracle and the reduced result must equal the single-rank J/K.
The benchmark's timing rule (max over ranks) is checked the same way."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import CGF


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, cgfs, D, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    cg = [CGF(d) for d in cgfs]
    J, K = O.jk_direct(cg, D, nthreads=1, stride=world, phase=rank)
    t = torch.tensor(np.stack([J, K]))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    ms = torch.tensor([10.0 * (rank + 1)], dtype=torch.float64)
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((t.numpy(), float(ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_partial_jk_allreduce(h2o_golden):
    from oracle import oracle as O
    cgfs = h2o_golden["cgfs"]
    D = np.array(h2o_golden["density"])
    Jr, Kr = O.jk_direct([CGF(d) for d in cgfs], D, nthreads=1)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, cgfs, D, q)) for r in range(2)]
    for p in procs:
        p.start()
    res, ms = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    np.testing.assert_allclose(res[0], Jr, atol=1e-13)
    np.testing.assert_allclose(res[1], Kr, atol=1e-13)
    assert ms == 20.0

"""Replica parallelism on CPU with the gloo backend (world size 2).

The hot path does not shard: every chain is a sequential Markov process and
the reference's MPI ranks never exchange data during Monte Carlo
(src/Main_PQMC.f90:373-443).  Each rank advances its own chains from
rank-dependent seeds; the only collectives are the timing barrier and the
max-over-ranks reduction of the step time (bench.py).  Checked here with the
oracle as the per-rank engine: ranks see different fields, a rank's result
does not depend on the other rank, and the reductions behave as the bench
uses them.
"""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from tests.helpers import epsocz_small


def _rank_main(rank, world, port, out_q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.rng import seed_words
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, seed=2 + rank)
    o = OracleChain(m, field=f, seed_words=seed_words(1000 + rank), meas=False)
    o.init_expkv()
    o.init_g(1)
    dist.barrier()
    o.sweep(1, 1)
    st = o.state()
    # max over ranks of a per-rank time, as bench.py reduces the step time
    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    acc = torch.tensor([float(st["positive_accept"])], dtype=torch.float64)
    gathered = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, acc)
    out_q.put((rank, float(t.item()), [float(x.item()) for x in gathered], o.field().copy(), st["positive_accept"]))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda x: x[0])
    (r0, t0, g0, f0, a0), (r1, t1, g1, f1, a1) = res
    assert t0 == t1 == 2.0                      # max over ranks
    assert g0 == g1 == [float(a0), float(a1)]   # every rank sees both counts
    assert not np.array_equal(f0, f1)           # independent replicas

    # a rank's chain is the same chain it would be alone
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.rng import seed_words
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, seed=3)
    o = OracleChain(m, field=f, seed_words=seed_words(1001), meas=False)
    o.init_expkv()
    o.init_g(1)
    o.sweep(1, 1)
    assert np.array_equal(o.field(), f1)

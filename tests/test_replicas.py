"""Multi-GPU form of the bench: independent replicas (one realisation per
rank, no data-path collective), job time = the slowest rank's.  Exercised
here with two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's own realisation: its seed table (the oracle, N = 16)
        from oracle import oracle as O
        from tests.common import bbks, make_cfg
        cfg = make_cfg(16, 100.0, bench.replica_seed(rank), 10.0, 8, "local_m8_L500_n128", 128)
        table = O.Oracle(cfg, *bbks()).seedtable().astype(np.int64)
        tables = [torch.zeros(16 * 16, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(tables, torch.from_numpy(table.ravel()))  # test-side check only
        slowest = bench.max_over_ranks(1.0 + 0.5 * rank)
        rate = bench.job_rate(world, 3, 1000, slowest)
        out.put((rank, slowest, rate, [t.numpy() for t in tables]))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    from oracle import oracle as O
    O.build()
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate, tables in res:
        assert slowest == 1.5  # max over ranks, on every rank
        assert rate == world * 3 * 1000 / 1.5  # all ranks' units over the slowest time
        assert not np.array_equal(tables[0], tables[1])  # independent realisations
    assert np.array_equal(res[0][3][1], res[1][3][1])


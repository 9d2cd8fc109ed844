"""The modal sum split over radial modes across ranks.

CPU (gloo, two ranks): each rank computes its share of the FP64 oracle's
regrouped accumulation for the r the library's partition gives it, and the
same reduce the GPU ranks use (modal_split.reduce_modal_share) yields the
unsplit non-Gaussian potential of the oracle's reference-structure loop
(main.c:564-1063) to 1e-12.  GPU: the shares of one realisation computed one
after another on one device add up to the unsplit fused potential."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from tests.common import bbks, make_cfg, table

CFG = dict(N=16, box=500.0, seed=7, fnl=100.0, tab="scalarI_m20_L1000_n1024", M=20, nmax=1024)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cfg():
    c = CFG
    return make_cfg(c["N"], c["box"], c["seed"], c["fnl"], c["M"], c["tab"], c["nmax"])


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from aarambam_gb300 import modal_split
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg = _cfg()
        alpha, x0 = table(cfg["table"], cfg["N_modes"])
        o = O.Oracle(cfg, *bbks())
        g = o.gauss()
        part = modal_split.partition(alpha, world)
        acc = o.modal_acc_regrouped(alpha, x0, g, r_on=(part == rank).astype(np.int32))
        n3 = float(cfg["Nmesh"]) ** 3
        gauss = torch.complex(torch.from_numpy(g[..., 0]), torch.from_numpy(g[..., 1]))
        share = gauss + cfg["Fnl"] / n3 * torch.complex(torch.from_numpy(acc[..., 0]), torch.from_numpy(acc[..., 1]))
        tot = modal_split.reduce_modal_share(gauss, share, root=0)
        out.put((rank, None if tot is None else (tot - gauss).numpy(), part))
    finally:
        dist.destroy_process_group()


def test_split_modal_sum_gloo():
    from aarambam_gb300 import _lib
    from oracle import oracle as O
    _lib.load(build_if_missing=True)
    O.build()
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in range(world)), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[1][1] is None  # only the root holds the total
    assert np.array_equal(res[0][2], res[1][2])  # every rank derives the same partition
    cfg = _cfg()
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    o = O.Oracle(cfg, *bbks())
    full = o.modal_acc(alpha, x0, o.gauss())
    want = cfg["Fnl"] / float(cfg["Nmesh"]) ** 3 * (full[..., 0] + 1j * full[..., 1])
    got = res[0][1]
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


def test_partition_balanced_and_complete():
    from aarambam_gb300 import modal_split
    alpha, _ = table("scalarI_m20_L1000_n1024", 20)
    M = alpha.shape[0]
    # product terms per target r (sorted triples, plus the counter-terms into r = 1 and 2)
    cnt = np.zeros(M, int)
    for p in range(M):
        for q in range(p, M):
            for r in range(q, M):
                cnt[r] += alpha[p, q, r] != 0
    if alpha[0, 1, 2] != 0:
        cnt[2] += 1
        cnt[1] += 1
    active = cnt > 0
    for nparts in (1, 2, 3, 4, 8):
        part = modal_split.partition(alpha, nparts)
        assert np.all((part >= 0) == active)
        assert part[active].max() < nparts
        loads = np.array([cnt[part == k].sum() for k in range(nparts)])
        assert loads.sum() == cnt.sum()
        assert loads.max() - loads.min() <= cnt.max()  # greedy largest-first bound


@pytest.mark.gpu
@pytest.mark.parametrize("N,nparts", [(32, 2), (64, 3), (256, 2)])
def test_split_shares_add_up_gpu(cuda, N, nparts):
    """On one GPU, the shares of all parts (each through the plan's own
    modal stage, NVRTC kernels re-specialised per part at 256^3) add up to
    the unsplit non-Gaussian potential to FP32 rounding.  Each share is read
    as (total - Gaussian) of an FP32 spectrum, so it carries the rounding of
    the total potential: bounded like the other parity tests (non-Gaussian
    part 1e-4, total 1e-6)."""
    from aarambam_gb300.ic import ICGenerator
    tab, M = "scalarI_m20_L1000_n1024", 20
    cfg = make_cfg(N, 1000.0, 5, 100.0, M, tab, 1024)
    g = ICGenerator(cfg, *table(tab, M), *bbks())
    g.stage("noise")
    gauss = g.spectrum()
    g.stage("modal")
    ng = (g.spectrum() - gauss).to(torch.complex128)
    tot = torch.zeros_like(ng)
    for k in range(nparts):
        g.set_modal_partition(k, nparts)
        g.stage("noise")
        g.stage("modal")
        tot += (g.spectrum() - gauss).to(torch.complex128)
    g.set_modal_partition(0, 1)
    err = float(torch.linalg.vector_norm(tot - ng) / torch.linalg.vector_norm(ng))
    err_tot = float(torch.linalg.vector_norm(tot - ng) / torch.linalg.vector_norm(gauss.to(torch.complex128) + ng))
    assert err < 1e-4
    assert err_tot < 1e-6

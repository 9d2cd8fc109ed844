"""The modal sum split over radial modes across ranks (one GPU per rank).

The regrouped modal potential acc = sum_r rho_r r2c(g_r) (the loop of
Aarambam/LPT/Basis/main.c:564-880, regrouped by linearity) is a sum of
independent terms once the Gaussian potential is known.  Every rank
regenerates the Gaussian potential from the seed (deterministic: no
broadcast), sums its own share of the r (`partition`: balanced by the number
of product terms per r), and one reduce of the non-Gaussian parts to the
root gives the unsplit potential there; the root then runs 2LPT and the
read-out.  (The reference distributes the same loop differently: x-slabs of
every field over MPI ranks, main.c:1556-1599.)  The collective is the
process group's (NCCL between GPUs, gloo on CPUs).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch
import torch.distributed as dist

from . import _lib


def partition(alpha: np.ndarray, nparts: int) -> np.ndarray:
    """Part of each radial mode r (int32 [M], -1 for an r without product
    terms), as the plans' aar_set_modal_partition uses it."""
    L = _lib.load()
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    M = a.shape[0]
    out = (C.c_int32 * M)()
    rc = L.aar_modal_partition(a.ctypes.data_as(C.POINTER(C.c_double)), M, int(nparts), out)
    if rc != _lib.AAR_OK:
        raise _lib.AarError(rc, "aar_modal_partition: bad arguments")
    return np.array(out[:], dtype=np.int32)


def reduce_modal_share(gauss: torch.Tensor, share: torch.Tensor, root: int = 0, group=None):
    """Sum over the ranks of (share - gauss), each rank's non-Gaussian part,
    added to the Gaussian spectrum on `root` (complex tensors of one shape on
    every rank).  Returns the total spectrum on the root, None elsewhere."""
    delta = (share - gauss).contiguous()
    dist.reduce(torch.view_as_real(delta), dst=root, op=dist.ReduceOp.SUM, group=group)
    if dist.get_rank(group) == root:
        return gauss + delta
    return None


def split_potential(gen, rank: int, world: int, root: int = 0, group=None) -> bool:
    """The modal potential of `gen`'s realisation computed by `world` ranks
    together; on the root the plan's spectrum is the total potential
    afterwards.  Returns True on the root."""
    gen.set_modal_partition(rank, world)
    gen.stage("noise")
    gauss = gen.spectrum()
    gen.stage("modal")
    share = gen.spectrum()
    total = reduce_modal_share(gauss, share, root, group)
    if total is None:
        return False
    gen.set_spectrum(total)
    return True


def split_run(gen, lagr: torch.Tensor, rank: int, world: int, root: int = 0, group=None, pos=None, vel=None):
    """One realisation made by `world` ranks: the split modal potential,
    then 2LPT and the read-out on the root.  Returns (pos, vel) on the root,
    None elsewhere."""
    if not split_potential(gen, rank, world, root, group):
        return None
    gen.stage("lpt")
    return gen.readout(lagr, pos, vel)

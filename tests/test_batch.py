"""Batches: several realisations (own seed, table, mode count) captured into
one CUDA graph give the same particles as running each plan alone."""
import pytest
import torch

from aarambam_gb300.ic import ICBatch, ICGenerator
from tests.common import bbks, make_cfg, table

pytestmark = pytest.mark.gpu

TEMPLATES = [("local_m6_L500_n256", 6), ("equil_m9_L500_n256", 9), ("scalarI_m10_L500_n256", 10),
             ("scalarI_m20_L500_n256_mu1p75", 20)]


def lattice(N, box, dev):
    g = torch.arange(N, device=dev, dtype=torch.float32) * (box / N)
    x, y, z = torch.meshgrid(g, g, g, indexing="ij")
    return torch.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], 1).contiguous()


def make_gens(N, n):
    gens = []
    for i in range(n):
        tab, M = TEMPLATES[i % len(TEMPLATES)]
        cfg = make_cfg(N, 500.0, 100 + i, 10.0 * (i + 1), M, tab, 256)
        gens.append(ICGenerator(cfg, *table(tab, M), *bbks()))
    return gens


def test_batch_graph_matches_single_runs(cuda):
    N, n = 64, 5
    gens = make_gens(N, n)
    lagr = [lattice(N, 500.0, cuda) for _ in range(n)]
    want = [g.run(l) for g, l in zip(gens, lagr)]
    torch.cuda.synchronize()
    b = ICBatch(gens)
    pos = [torch.full_like(l, float("nan")) for l in lagr]
    vel = [torch.full_like(l, float("nan")) for l in lagr]
    for _ in range(2):  # capture, then replay
        b.run(lagr, pos, vel)
        torch.cuda.synchronize()
        for i in range(n):
            assert torch.equal(pos[i], want[i][0]) and torch.equal(vel[i], want[i][1]), i
    assert b.launches == sum(g.launches for g in gens)
    # a changed seed makes the graph stale: it is captured again
    gens[1].set_seed(777)
    want1 = gens[1].run(lagr[1])
    b.run(lagr, pos, vel)
    torch.cuda.synchronize()
    assert torch.equal(pos[1], want1[0]) and torch.equal(vel[1], want1[1])
    assert torch.equal(pos[0], want[0][0])
    b.close()


def test_batch_graph_with_runtime_row_kernel(cuda):
    # 256^3: the modal rows run the NVRTC-specialised kernel inside the graph
    N, n = 256, 2
    gens = make_gens(N, n)
    assert all(g.jit_status == "on" for g in gens)
    lagr = [lattice(N, 500.0, cuda) for _ in range(n)]
    want = [g.run(l) for g, l in zip(gens, lagr)]
    torch.cuda.synchronize()
    b = ICBatch(gens)
    pos = [torch.empty_like(l) for l in lagr]
    vel = [torch.empty_like(l) for l in lagr]
    for _ in range(2):
        b.run(lagr, pos, vel)
        torch.cuda.synchronize()
        for i in range(n):
            assert torch.equal(pos[i], want[i][0]) and torch.equal(vel[i], want[i][1]), i
    b.close()


def test_batch_rejects_bad_arrays(cuda):
    gens = make_gens(32, 2)
    b = ICBatch(gens)
    lagr = [lattice(32, 500.0, cuda) for _ in range(2)]
    with pytest.raises(ValueError):
        b.run(lagr, lagr[:1], lagr)
    b.close()


def test_batch_recaptured_after_autotune(cuda):
    """aar_autotune reloads the plan's NVRTC module for its candidates, so a
    batch graph captured before it must be captured again whatever the
    tuner's outcome; here the tuner returns an error (its report buffer is
    too small) after it has tried every candidate."""
    import ctypes as C

    from aarambam_gb300._lib import AAR_ERR_ARG
    N, n = 64, 2
    gens = make_gens(N, n)
    for g in gens:
        assert g.set_jit(2) == "on"
    lagr = [lattice(N, 500.0, cuda) for _ in range(n)]
    want = [[t.clone() for t in g.run(l)] for g, l in zip(gens, lagr)]
    b = ICBatch(gens)
    pos = [torch.empty_like(l) for l in lagr]
    vel = [torch.empty_like(l) for l in lagr]
    b.run(lagr, pos, vel)
    torch.cuda.synchronize()
    small = C.create_string_buffer(8)
    rc = gens[0].L.aar_autotune(gens[0].h, small, len(small), gens[0]._stream())
    assert rc == AAR_ERR_ARG
    torch.cuda.synchronize()
    # the tuner may have chosen another row kernel: compare with single runs now
    want = [[t.clone() for t in g.run(l)] for g, l in zip(gens, lagr)]
    torch.cuda.synchronize()
    b.run(lagr, pos, vel)
    torch.cuda.synchronize()
    for i in range(n):
        assert torch.equal(pos[i], want[i][0]) and torch.equal(vel[i], want[i][1]), i
    b.close()

"""Full-size checks (the bench workloads' grids) through size-independent
properties: the seed table bit-exact at 1024^3, the transforms' round trip,
the white-noise spectrum's structure, and the fused FP32 particles against
the plain FP64 GPU form at 512^3."""
import numpy as np
import pytest
import torch

from aarambam_gb300.ic import ICGenerator
from oracle import oracle as O
from tests.common import bbks, make_cfg, table

pytestmark = pytest.mark.gpu


def gen(N, tab="local_m8_L500_n128", M=8, nmax=None, **kw):
    cfg = make_cfg(N, 1000.0, 2026, 100.0, M, tab, nmax or max(N, 128), **kw)
    return ICGenerator(cfg, *table(tab, M), *bbks()), cfg


def test_seedtable_bit_exact_1024(cuda):
    g, cfg = gen(1024)
    got = g.seedtable().cpu().numpy().view(np.uint32)
    want = O.Oracle(cfg, *bbks()).seedtable()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("N", [512, 1024])
def test_transform_round_trip(cuda, N):
    g, _ = gen(N)
    x = torch.randn((N, N, N), generator=torch.Generator(device="cuda").manual_seed(N), device=cuda)
    y = g.c2r(g.r2c(x))
    # c2r(r2c(x)) = N^3 x with FFTW's unnormalised conventions
    err = torch.linalg.vector_norm(y / float(N) ** 3 - x) / torch.linalg.vector_norm(x)
    assert float(err) < 2e-6


def test_white_noise_structure_1024(cuda):
    g, cfg = gen(1024)
    N = 1024
    g.stage("noise")
    X = g.spectrum()
    # no Nyquist index on x or y, no kz = N/2 plane, no DC (main.c:405-408)
    assert int(torch.count_nonzero(X[N // 2])) == 0 and int(torch.count_nonzero(X[:, N // 2])) == 0
    assert int(torch.count_nonzero(X[:, :, N // 2])) == 0 and complex(X[0, 0, 0]) == 0
    # the kz = 0 plane is Hermitian, written as value and conjugate (main.c:463-520)
    P = X[:, :, 0]
    idx = (-torch.arange(N, device=cuda)) % N
    Q = P[idx][:, idx].conj()
    assert torch.equal(P, Q)
    # cube cut at Nsample/2 = N/2 keeps every other cell: the fraction of zeros
    # in the interior is the count of the skipped indices only
    assert int(torch.count_nonzero(X[1:N // 2, 1:N // 2, 1:N // 2])) == (N // 2 - 1) ** 3


def test_fused_vs_plain_fp64_512(cuda):
    N = 512
    tab, M = "scalarI_m12_L1000_n512", 12
    cfg = make_cfg(N, 1000.0, 1234, 100.0, M, tab, 512)
    a, x0 = table(tab, M)
    k, t = bbks()
    g = torch.arange(N, device=cuda, dtype=torch.float32) * (1000.0 / N)
    gx, gy, gz = torch.meshgrid(g, g, g, indexing="ij")
    lagr = torch.stack([gx.reshape(-1), gy.reshape(-1), gz.reshape(-1)], 1).contiguous()
    del gx, gy, gz
    gf = ICGenerator(cfg, a, x0, k, t)
    pf, _ = gf.run(lagr)
    del gf
    torch.cuda.empty_cache()
    gp = ICGenerator(cfg, a, x0, k, t, precision="fp64")
    pp, _ = gp.run(lagr)
    del gp
    torch.cuda.empty_cache()

    def dspl(p):
        d = p.double() - lagr.double()
        return d - 1000.0 * torch.round(d / 1000.0)
    want = dspl(pp)
    err = torch.linalg.vector_norm(dspl(pf) - want) / torch.linalg.vector_norm(want)
    assert float(err) < 1e-5


def test_fused_vs_plain_fp64_1024(cuda):
    """The 1024^3 bench workload (20-mode ScalarI table): fused FP32 particles
    through the NVRTC row kernel and through the generic one, against the
    plain FP64 GPU form.  Rows of N = 1024 fold the radix-2 step of the
    half-length transform into the c2r pre- and r2c post-steps, so this is
    the one size that runs those steps."""
    N = 1024
    tab, M = "scalarI_m20_L1000_n1024", 20
    cfg = make_cfg(N, 1000.0, 77, 100.0, M, tab, 1024)
    a, x0 = table(tab, M)
    k, t = bbks()
    g = torch.arange(N, device=cuda, dtype=torch.float32) * (1000.0 / N)
    gx, gy, gz = torch.meshgrid(g, g, g, indexing="ij")
    lagr = torch.stack([gx.reshape(-1), gy.reshape(-1), gz.reshape(-1)], 1).contiguous()
    del gx, gy, gz
    gf = ICGenerator(cfg, a, x0, k, t)
    assert gf.jit_status == "on"
    pj, _ = gf.run(lagr)
    gf.set_jit(0)
    pg, _ = gf.run(lagr)
    gf.close()
    del gf
    torch.cuda.empty_cache()
    gp = ICGenerator(cfg, a, x0, k, t, precision="fp64")
    pp, _ = gp.run(lagr)
    gp.close()
    del gp
    torch.cuda.empty_cache()

    def rel(p):
        num = den = 0.0
        for s in range(0, lagr.shape[0], 1 << 25):
            sl = slice(s, s + (1 << 25))
            L = lagr[sl].double()
            w = pp[sl].double() - L
            w -= 1000.0 * torch.round(w / 1000.0)
            d = p[sl].double() - L
            d -= 1000.0 * torch.round(d / 1000.0)
            num += float(torch.sum((d - w) ** 2))
            den += float(torch.sum(w ** 2))
        return (num / den) ** 0.5
    assert rel(pj) < 1e-5
    assert rel(pg) < 1e-5

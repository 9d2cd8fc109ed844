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


def _delta(psi1, box):
    """delta = -div psi1 (spectral derivative, FP64), psi1 three [N, N, N] fields."""
    N = psi1[0].shape[0]
    dev = psi1[0].device
    k = 2 * np.pi / box * torch.fft.fftfreq(N, 1.0 / N, dtype=torch.float64, device=dev)
    kz = 2 * np.pi / box * torch.arange(N // 2 + 1, dtype=torch.float64, device=dev)
    ks = [k[:, None, None], k[None, :, None], kz[None, None, :]]
    d = sum(1j * ks[a] * torch.fft.rfftn(psi1[a].double()) for a in range(3))
    return -torch.fft.irfftn(d, s=(N, N, N))


def _rel(a, b):
    num = sum(float(torch.sum((x.double() - y.double()) ** 2)) for x, y in zip(a, b))
    den = sum(float(torch.sum(y.double() ** 2)) for y in b)
    return (num / den) ** 0.5


def test_precision_config_512(cuda):
    """The precision configuration at its stated size: 512^3, Box 1000,
    ScalarI mass 1, 12 modes.  Relative RMS of delta = -div psi1, psi1 and
    psi2 of the fused FP32 form against the plain FP64 GPU form's FP64
    fields (that form is pinned to the FP64 oracle by
    test_plain_fp64_fields_vs_oracle), and of the particle displacement."""
    N, box = 512, 1000.0
    tab, M = "scalarI_m12_L1000_n512", 12
    cfg = make_cfg(N, box, 1234, 100.0, M, tab, 512)
    a, x0 = table(tab, M)
    k, t = bbks()
    g = torch.arange(N, device=cuda, dtype=torch.float32) * (box / N)
    gx, gy, gz = torch.meshgrid(g, g, g, indexing="ij")
    lagr = torch.stack([gx.reshape(-1), gy.reshape(-1), gz.reshape(-1)], 1).contiguous()
    del gx, gy, gz
    gf = ICGenerator(cfg, a, x0, k, t)
    pf, _ = gf.run(lagr)
    ff = [gf.field(i) for i in range(6)]
    gf.close()
    del gf
    torch.cuda.empty_cache()
    gp = ICGenerator(cfg, a, x0, k, t, precision="fp64")
    pp, _ = gp.run(lagr)
    fp = [gp.field(i) for i in range(6)]
    gp.close()
    del gp
    torch.cuda.empty_cache()
    e_psi1 = _rel(ff[:3], fp[:3])
    e_psi2 = _rel(ff[3:], fp[3:])
    e_delta = _rel([_delta(ff[:3], box)], [_delta(fp[:3], box)])

    def dspl(p):
        d = p.double() - lagr.double()
        return d - box * torch.round(d / box)
    e_disp = _rel([dspl(pf)], [dspl(pp)])
    print(f"precision 512^3 M=12: delta {e_delta:.3e} psi1 {e_psi1:.3e} psi2 {e_psi2:.3e} displacement {e_disp:.3e}")
    assert e_psi1 < 1e-5 and e_delta < 1e-5
    assert e_psi2 < 2e-4
    assert e_disp < 1e-5


def test_modal_potential_vs_plain_fp64_512(cuda):
    """The modal non-Gaussian potential at 512^3 (12-mode ScalarI table),
    where the filter x pass runs its 32-values-per-lane form (field filters
    evaluated per cell, mirrored by shuffle): fused FP32 total potential and
    its non-Gaussian part against the plain FP64 GPU form's."""
    N, box = 512, 1000.0
    tab, M = "scalarI_m12_L1000_n512", 12
    cfg = make_cfg(N, box, 99, 100.0, M, tab, 512)
    a, x0 = table(tab, M)
    k, t = bbks()
    gf = ICGenerator(cfg, a, x0, k, t)
    gf.stage("noise")
    gauss = gf.spectrum().to(torch.complex128)
    gf.stage("modal")
    tot = gf.spectrum().to(torch.complex128)
    gf.close()
    del gf
    torch.cuda.empty_cache()
    import ctypes as C
    gp = ICGenerator(cfg, a, x0, k, t, precision="fp64")
    ref_gauss = torch.empty((N, N, N // 2 + 1), dtype=torch.complex128, device=cuda)
    assert gp.L.aar_gaussian_spectrum_noalloc(gp.h, ref_gauss.data_ptr(),
                                              C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    lagr = torch.zeros((1, 3), dtype=torch.float32, device=cuda)
    gp.run(lagr)
    ref_tot = gp.spectrum()
    gp.close()
    del gp
    torch.cuda.empty_cache()
    ng = tot - gauss
    ref_ng = ref_tot - ref_gauss
    e_ng = float(torch.linalg.vector_norm(ng - ref_ng) / torch.linalg.vector_norm(ref_ng))
    e_tot = float(torch.linalg.vector_norm(tot - ref_tot) / torch.linalg.vector_norm(ref_tot))
    print(f"modal 512^3 M=12 vs plain FP64: non-Gaussian part {e_ng:.3e}, total {e_tot:.3e}")
    assert e_ng < 2e-4
    assert e_tot < 1e-6


def test_run_lattice_1024(cuda):
    """The 1024^3 bench workload through aar_run_lattice (64^3 lattice glass
    tiled 16 times, read-out fused into the folded displacement rows): the
    general glass read-out's particles to float rounding (the grid value
    under each particle against the FP32 two-float coordinate's ~1e-12
    neighbour weights)."""
    from aarambam_gb300 import gadget
    N = 1024
    tab, M = "scalarI_m20_L1000_n1024", 20
    cfg = make_cfg(N, 1000.0, 12, 100.0, M, tab, 1024)
    gen = ICGenerator(cfg, *table(tab, M), *bbks())
    glass = torch.from_numpy(gadget.lattice_glass(64, 100.0)).cuda()
    pos_g, vel_g, _ = gen.run_glass(glass, 100.0, 16)
    pos = torch.full_like(pos_g, float("nan"))
    vel = torch.full_like(vel_g, float("nan"))
    gen.run_lattice(64, 100.0, 16, pos, vel)
    same = float((pos == pos_g).all(1).float().mean())
    print(f"lattice read-out at 1024^3: {100 * same:.4f} % of particles bit-identical to the general read-out")
    d = (pos.double() - pos_g.double()).abs()
    assert bool(torch.all(torch.minimum(d, 1000.0 - d) <= 1e-4))
    torch.testing.assert_close(vel, vel_g, rtol=1e-6, atol=1e-6 * float(vel_g.abs().max()))

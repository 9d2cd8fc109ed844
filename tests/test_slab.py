"""The slab form (AAR_SLAB_FP32): the FP32 path streamed over x-slabs, for
grids whose fused fields do not fit one GPU.  Checked against the fused form
(power-of-two grids; the same FP32 arithmetic, another schedule and FFT) and
against the plain FP64 regrouped form on grids the fused form does not take
(N = 48, 96: radix-3 lines, as at 1536^3).  Tolerances are relative RMS
errors, stated per test."""
import numpy as np
import pytest
import torch

from tests.common import bbks, make_cfg, periodic_delta, rel_rms, table

pytestmark = pytest.mark.gpu


def gen_for(cfg, precision="fp32", **kw):
    from aarambam_gb300.ic import ICGenerator
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    k, t = bbks()
    return ICGenerator(cfg, alpha, x0, k, t, precision=precision, **kw)


def lattice(N, box, dev):
    g = np.arange(N, dtype=np.float64) * (box / N)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    return torch.from_numpy(np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(np.float32)).to(dev)


def run_all(gen, lagr):
    pos, vel = gen.run(lagr)
    spec = gen.spectrum().cpu().numpy()
    f = np.stack([gen.field(i).double().cpu().numpy() for i in range(6)])
    return pos, vel, spec, f


@pytest.mark.parametrize("N,S,box,M,tab", [(32, 4, 500.0, 10, "scalarI_m10_L500_n256"),
                                           (64, 8, 1000.0, 12, "scalarI_m12_L1000_n512"),
                                           (64, 2, 500.0, 8, "local_m8_L500_n128"),
                                           (128, 4, 1000.0, 20, "scalarI_m20_L1000_n1024"),
                                           (64, 1, 500.0, 10, "scalarI_m10_L500_n256")])
def test_slab_matches_fused(cuda, N, S, box, M, tab):
    """Slab form against the fused form on the same realisation: total
    potential to 1e-6, psi1 to 2e-6, psi2 (FP32 cancellation in the source)
    to 1e-4, velocities to 2e-6; particle displacements (Pos - q, with Pos
    rounded to float at |Pos| up to Box) to 1e-5, the float position
    rounding of the two forms."""
    cfg = make_cfg(N, box, 4242, 100.0, M, tab, max(N, 256))
    lagr = lattice(N, box, cuda)
    pf, vf, sf, ff = run_all(gen_for(cfg), lagr)
    g = gen_for(cfg, precision="slab_fp32", nslab=S)
    ps, vs, ss, fs = run_all(g, lagr)
    e_phi = rel_rms(ss, sf)
    e1, e2 = rel_rms(fs[:3], ff[:3]), rel_rms(fs[3:], ff[3:])
    lg = lagr.cpu().numpy()
    ed = rel_rms(periodic_delta(ps.cpu().numpy(), lg, box), periodic_delta(pf.cpu().numpy(), lg, box))
    ev = rel_rms(vs.cpu().numpy(), vf.cpu().numpy())
    print(f"N={N} S={S}: phi {e_phi:.2e} psi1 {e1:.2e} psi2 {e2:.2e} disp {ed:.2e} vel {ev:.2e}")
    assert e_phi < 1e-6
    assert e1 < 2e-6
    assert e2 < 1e-4
    assert ed < 1e-5 and ev < 2e-6


def test_slab_256_matches_unslabbed(cuda):
    """The slab schedule at 256^3 (S = 8, 10 modes) against the unslabbed
    fused form: the total potential agrees to 1e-6."""
    cfg = make_cfg(256, 500.0, 99, 100.0, 10, "scalarI_m10_L500_n256", 256)
    a = gen_for(cfg)
    a.stage("noise")
    a.stage("modal")
    want = a.spectrum().cpu().numpy()
    del a
    torch.cuda.empty_cache()
    g = gen_for(cfg, precision="slab_fp32", nslab=8)
    g.run(lattice(64, 500.0, cuda))  # any particles: the potential is what is compared
    got = g.spectrum().cpu().numpy()
    e = rel_rms(got, want)
    print(f"256^3 S=8: phi {e:.2e}")
    assert e < 1e-6


@pytest.mark.parametrize("N,S,box", [(48, 3, 300.0), (96, 4, 600.0), (96, 12, 600.0)])
def test_slab_non_power_of_two_vs_plain_fp64(cuda, N, S, box):
    """Grids with a factor 3 (the 1536^3 case's radix): the slab form against
    the plain FP64 regrouped form (pinned to the oracle) -- total potential
    to 1e-6, psi1 to 1e-5, psi2 to 1e-4, particle displacements to 1e-5."""
    cfg = make_cfg(N, box, 77, 100.0, 12, "scalarI_m12_L1000_n512", 512)
    lagr = lattice(N, box, cuda)
    pp, vp, sp, fp = run_all(gen_for(cfg, precision="fp64_regrouped"), lagr)
    ps, vs, ss, fs = run_all(gen_for(cfg, precision="slab_fp32", nslab=S), lagr)
    e_phi = rel_rms(ss, sp)
    e1, e2 = rel_rms(fs[:3], fp[:3]), rel_rms(fs[3:], fp[3:])
    lg = lagr.cpu().numpy()
    ed = rel_rms(periodic_delta(ps.cpu().numpy(), lg, box), periodic_delta(pp.cpu().numpy(), lg, box))
    print(f"N={N} S={S}: phi {e_phi:.2e} psi1 {e1:.2e} psi2 {e2:.2e} disp {ed:.2e}")
    assert e_phi < 1e-6
    assert e1 < 1e-5
    assert e2 < 1e-4
    assert ed < 1e-5


@pytest.mark.parametrize("kw", [dict(SphereMode=1, Nsample=40), dict(Fnl=0.0), dict(PhaseFlip=1, FixedAmplitude=1),
                                dict(A_res=0.3, w_res=12.0, phi_res=0.4, WhichSpectrum=2)],
                         ids=["sphere_cut", "fnl0", "flip_fixed", "resbasis"])
def test_slab_options_vs_plain_fp64(cuda, kw):
    """The slab form under the parameter-file options the other forms take
    (sphere cut below Nyquist, no non-Gaussian term, phase flip with fixed
    amplitude, the 2LPTResBasis oscillation) on a 48^3 grid, against the
    plain FP64 regrouped form: potential to 1e-6, psi1 to 1e-5, particle
    displacements to 1e-5."""
    base = dict(Fnl=100.0)
    base.update(kw)
    fnl = base.pop("Fnl")
    cfg = make_cfg(48, 300.0, 13, fnl, 10, "scalarI_m10_L500_n256", 256, **base)
    lagr = lattice(48, 300.0, cuda)
    pp, _, sp, fp = run_all(gen_for(cfg, precision="fp64_regrouped"), lagr)
    ps, _, ss, fs = run_all(gen_for(cfg, precision="slab_fp32", nslab=4), lagr)
    e_phi, e1 = rel_rms(ss, sp), rel_rms(fs[:3], fp[:3])
    lg = lagr.cpu().numpy()
    ed = rel_rms(periodic_delta(ps.cpu().numpy(), lg, 300.0), periodic_delta(pp.cpu().numpy(), lg, 300.0))
    print(f"{kw}: phi {e_phi:.2e} psi1 {e1:.2e} disp {ed:.2e}")
    assert e_phi < 1e-6 and e1 < 1e-5 and ed < 1e-5


def test_slab_read_out_entry_points(cuda):
    """The slab form leaves the six real displacement fields in the plan's
    layout: aar_run_lattice, aar_run_glass and the host-glass entry point
    read them out identically."""
    from aarambam_gb300 import gadget
    N, g, box = 48, 16, 300.0
    cfg = make_cfg(N, box, 5, 100.0, 8, "local_m8_L500_n128", 128)
    gen = gen_for(cfg, precision="slab_fp32", nslab=6)
    tile = N // g
    glass = torch.from_numpy(gadget.lattice_glass(g, 100.0)).cuda()
    pg, vg, ig = gen.run_glass(glass, 100.0, tile)
    pl = torch.empty_like(pg)
    vl = torch.empty_like(vg)
    il = torch.zeros_like(ig)
    gen.run_lattice(g, 100.0, tile, pl, vl, il)
    assert torch.equal(pl, pg) and torch.equal(vl, vg) and torch.equal(il, ig)
    hp, hv, hi = gen.run_glass_host(gadget.lattice_glass(g, 100.0), 100.0, tile)
    assert np.array_equal(hp, pg.cpu().numpy()) and np.array_equal(hv, vg.cpu().numpy())
    assert np.array_equal(hi, ig.cpu().numpy())


def test_slab_host_read_out(cuda):
    """Page-locked host outputs (how the 1536^3 run returns its particles):
    the read-out kernel writes them over the host link, bit-identical to the
    read-out into device buffers (a glass tiled to 12^3 x 16^3 particles on
    a 48^3 grid, off the grid points)."""
    from aarambam_gb300 import gadget
    N, g, tile, box = 48, 16, 12, 300.0
    cfg = make_cfg(N, box, 8, 100.0, 8, "local_m8_L500_n128", 128)
    gen = gen_for(cfg, precision="slab_fp32", nslab=4)
    n = g ** 3 * tile ** 3
    pd = torch.empty((n, 3), dtype=torch.float32, device=cuda)
    vd = torch.empty_like(pd)
    idd = torch.zeros(n, dtype=torch.int32, device=cuda)
    gen.run_lattice(g, 100.0, tile, pd, vd, idd)
    ph = torch.full((n, 3), float("nan"), dtype=torch.float32).pin_memory()
    vh = torch.full((n, 3), float("nan"), dtype=torch.float32).pin_memory()
    ih = torch.zeros(n, dtype=torch.int32).pin_memory()
    gen.run_lattice(g, 100.0, tile, ph, vh, ih)
    torch.cuda.synchronize()
    assert torch.equal(ph, pd.cpu()) and torch.equal(vh, vd.cpu()) and torch.equal(ih, idd.cpu())


def test_slab_memory(cuda):
    """Device memory of a slab plan: the potential, max(2F + (M + R) F_s,
    7F + 6 F_s) and the FFT work area (F one plan field, F_s one slab
    field), well below the fused plan's max(M, 9) + 1 fields."""
    from aarambam_gb300.ic import ICGenerator  # noqa: F401
    N, S, M = 128, 8, 20
    cfg = make_cfg(N, 1000.0, 1, 100.0, M, "scalarI_m20_L1000_n1024", 1024)
    alpha, _ = table(cfg["table"], M)
    rs = {r for p in range(M) for q in range(p, M) for r in range(q, M) if alpha[p, q, r] != 0}
    if alpha[0, 1, 2] != 0:  # the counter-terms write g_1 and g_2
        rs |= {1, 2}
    R = len(rs)
    g = gen_for(cfg, precision="slab_fp32", nslab=S)
    g.prepare()
    HP = ((N // 2 + 1) + 7) // 8 * 8
    F, Fs = 8 * N * N * HP, 8 * (N // S) * N * (N // 2 + 1)
    fields = F + max(2 * F + (M + R) * Fs, 7 * F + 6 * Fs)
    assert fields <= g.device_bytes <= fields + 0.5 * F + (64 << 20)
    fused = gen_for(cfg)
    fused.prepare()
    fused.run(lattice(16, 1000.0, cuda))
    assert g.device_bytes < 0.5 * fused.device_bytes


def test_slab_argument_errors(cuda):
    from aarambam_gb300._lib import AarError
    cfg = make_cfg(48, 300.0, 1, 10.0, 8, "local_m8_L500_n128", 128)
    with pytest.raises(AarError, match="nslab"):
        gen_for(cfg, precision="slab_fp32", nslab=5)
    with pytest.raises(AarError, match="nslab"):
        gen_for(cfg, precision="slab_fp32", nslab=48)
    cfg2 = make_cfg(50, 300.0, 1, 10.0, 8, "local_m8_L500_n128", 128)
    with pytest.raises(AarError, match="multiple of 4"):
        gen_for(cfg2, precision="slab_fp32", nslab=2)

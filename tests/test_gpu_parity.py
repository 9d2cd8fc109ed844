"""Parity of the CUDA path (through the C ABI) with the FP64 oracle and with
the reference's own outputs.  Bit-exact: seed table, the zero pattern of the
Gaussian spectrum (Nyquist / DC / cut / Hermitian fill).  Tolerances (FP32
arithmetic against FP64): stated per test."""
import functools

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.common import (CASES, bbks, lattice_lagrangian, load_case, make_cfg, periodic_delta, rel_rms, table)

pytestmark = pytest.mark.gpu


def gen_for(cfg, precision="fp32", **kw):
    from aarambam_gb300.ic import ICGenerator
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    k, t = bbks()
    return ICGenerator(cfg, alpha, x0, k, t, precision=precision, **kw)


@functools.lru_cache(maxsize=None)
def oracle_run(key):
    cfg = dict(key)
    k, t = bbks()
    o = O.Oracle(cfg, k, t)
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    gn, tile = cfg.get("glass_n", cfg["Nmesh"]), cfg.get("GlassTileFac", 1)
    lagr = lattice_lagrangian(o, gn, tile)
    r = o.run(alpha, x0, lagr)
    r["lagr"] = lagr
    return r


def key(cfg):
    return tuple(sorted(cfg.items()))


SMALL = [
    make_cfg(16, 500.0, 1234, 10.0, 8, "local_m8_L500_n128", 128),
    make_cfg(32, 500.0, 4321, 100.0, 10, "scalarI_m10_L500_n256", 256, Nsample=24, PhaseFlip=1),
    make_cfg(32, 1000.0, 7, 100.0, 12, "scalarI_m12_L1000_n512", 512, SphereMode=1, Nsample=28),
    make_cfg(64, 500.0, 99, -50.0, 8, "local_m8_L500_n128", 128, FixedAmplitude=1),
    make_cfg(128, 500.0, 1234, 10.0, 8, "local_m8_L500_n128", 128),
]


@pytest.mark.parametrize("N,seed", [(16, 1234), (32, 4321), (64, 7), (128, 1), (256, 99), (512, 2024)])
def test_seedtable_bit_exact(cuda, N, seed):
    cfg = make_cfg(N, 500.0, seed, 10.0, 8, "local_m8_L500_n128", max(N, 128))
    g = gen_for(cfg)
    got = g.seedtable().cpu().numpy().view(np.uint32)
    k, t = bbks()
    want = O.Oracle(cfg, k, t).seedtable()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("cfg", SMALL[:4], ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_gaussian_spectrum(cuda, cfg):
    g = gen_for(cfg)
    g.stage("noise")
    got = g.spectrum().cpu().numpy()
    k, t = bbks()
    ref = O.Oracle(cfg, k, t).gauss()
    ref = ref[..., 0] + 1j * ref[..., 1]
    # exactly the same cells are set (skips after the draws, cut, Hermitian k=0 plane)
    assert np.array_equal(got != 0, ref != 0)
    # FP32 amplitude / phase from the bit-exact uniforms: per-cell relative error
    nz = ref != 0
    relerr = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    assert relerr.max() < 2e-6
    assert rel_rms(got, ref) < 3e-7


@pytest.mark.parametrize("cfg", SMALL[:4], ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_noise_blocks_match_one_draw(cuda, cfg, monkeypatch):
    """The noise kernel's six-cell blocks per generator refill give the
    same spectrum, bit for bit, as drawing every column one uniform at a
    time (the path a block with a zero U2 takes), FP32 and FP64 amplitude."""
    for fp64 in (False, True):
        g = gen_for(cfg, noise_fp64=fp64)
        g.stage("noise")
        fast = g.spectrum().cpu().numpy()
        monkeypatch.setenv("AAR_NOISE_ONE_DRAW", "1")
        h = gen_for(cfg, noise_fp64=fp64)
        monkeypatch.delenv("AAR_NOISE_ONE_DRAW")
        h.stage("noise")
        assert np.array_equal(h.spectrum().cpu().numpy(), fast)


@pytest.mark.parametrize("N", [16, 32, 64, 128])
def test_transforms_match_numpy(cuda, N):
    cfg = make_cfg(N, 500.0, 1, 10.0, 8, "local_m8_L500_n128", 128)
    g = gen_for(cfg)
    rng = np.random.default_rng(N)
    X = (rng.standard_normal((N, N, N // 2 + 1)) + 1j * rng.standard_normal((N, N, N // 2 + 1))).astype(np.complex64)
    y = g.c2r(torch.from_numpy(X).cuda()).cpu().numpy()
    yr = np.fft.irfftn(X.astype(np.complex128), s=(N, N, N), axes=(0, 1, 2)) * N**3
    assert rel_rms(y, yr) < 1e-6
    x = rng.standard_normal((N, N, N)).astype(np.float32)
    c = g.r2c(torch.from_numpy(x).cuda()).cpu().numpy()
    cr = np.fft.rfftn(x.astype(np.float64))
    assert rel_rms(c, cr) < 1e-6
    assert g.launches == 3


@pytest.mark.parametrize("cfg", SMALL, ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_nongaussian_potential(cuda, cfg):
    r = oracle_run(key(cfg))
    g = gen_for(cfg)
    g.stage("noise")
    gauss = g.spectrum().cpu().numpy().astype(np.complex128)
    g.stage("modal")
    tot = g.spectrum().cpu().numpy().astype(np.complex128)
    ref_tot = r["total"][..., 0] + 1j * r["total"][..., 1]
    ref_g = r["gauss"][..., 0] + 1j * r["gauss"][..., 1]
    N = cfg["Nmesh"]
    # the non-Gaussian part on its own: (total - gauss) N^3 / Fnl = acc
    ng = (tot - gauss) * N**3 / cfg["Fnl"]
    ref_ng = (ref_tot - ref_g) * N**3 / cfg["Fnl"]
    assert rel_rms(ng, ref_ng) < 2e-4
    assert rel_rms(tot, ref_tot) < 1e-6


@pytest.mark.parametrize("cfg", SMALL, ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_displacement_fields(cuda, cfg):
    r = oracle_run(key(cfg))
    g = gen_for(cfg)
    g.stage("noise")
    g.stage("modal")
    g.stage("lpt")
    # ZA fields to 1e-5; the 2LPT fields carry the FP32 rounding of the
    # Hessians through the cancelling source S = d00 (d11 + d22) + ... (their
    # weight in the displacement is 3/7 psi2 / N^3, about 1% at z = 49)
    for which in range(6):
        got = g.field(which).cpu().numpy()
        tol = 1e-5 if which < 3 else 2e-4
        assert rel_rms(got, r["disp"][which]) < tol, which


@pytest.mark.parametrize("cfg", SMALL, ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_particles_vs_oracle(cuda, cfg):
    r = oracle_run(key(cfg))
    g = gen_for(cfg)
    lagr = torch.from_numpy(r["lagr"]).cuda()
    pos, vel = g.run(lagr)
    pos, vel = pos.cpu().numpy(), vel.cpu().numpy()
    d_gpu = periodic_delta(pos, r["lagr"], cfg["Box"])
    d_ref = periodic_delta(r["pos"], r["lagr"], cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-5
    assert rel_rms(vel, r["vel"]) < 1e-5
    assert g.launches > 5


@pytest.mark.parametrize("name", [c for c in CASES if c != "local_n24"])
def test_particles_vs_reference_outputs(cuda, name):
    """Against the reference executable's own snapshot (tests/golden/ref)."""
    cfg, z = load_case(name)
    g = gen_for(cfg)
    k, t = bbks()
    o = O.Oracle(cfg, k, t)
    lagr = lattice_lagrangian(o, cfg["glass_n"], cfg["GlassTileFac"])
    pos, vel = g.run(torch.from_numpy(lagr).cuda())
    d_gpu = periodic_delta(pos.cpu().numpy(), lagr, cfg["Box"])
    d_ref = periodic_delta(z["pos"], lagr, cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-5
    assert rel_rms(vel.cpu().numpy(), z["vel"]) < 1e-5


def test_run_glass_matches_run(cuda):
    from aarambam_gb300 import gadget
    cfg, z = load_case("local_n32")
    g = gen_for(cfg)
    glass = gadget.lattice_glass(cfg["glass_n"], 100.0)
    pos_g, vel_g, ids = g.run_glass(torch.from_numpy(glass).cuda(), 100.0, cfg["GlassTileFac"])
    k, t = bbks()
    lagr = lattice_lagrangian(O.Oracle(cfg, k, t), cfg["glass_n"], cfg["GlassTileFac"])
    pos, vel = g.run(torch.from_numpy(lagr).cuda())
    assert torch.equal(pos_g, pos) and torch.equal(vel_g, vel)
    assert np.array_equal(ids.cpu().numpy(), z["ids"])


def test_random_glass_vs_oracle(cuda):
    """A glass that is not a lattice (uniform random positions, tiled 2^3
    times): trilinear weights of every corner in play (read_glass.c:129-214,
    main.c:1440-1516)."""
    cfg = dict(SMALL[0])
    rng = np.random.default_rng(11)
    glass = rng.uniform(0, 100.0, (3000, 3)).astype(np.float32)
    k, t = bbks()
    o = O.Oracle(cfg, k, t)
    lagr = o.tile_glass(glass, 100.0, 2)
    r = o.run(*table(cfg["table"], cfg["N_modes"]), lagr)
    g = gen_for(cfg)
    pos, vel, ids = g.run_glass(torch.from_numpy(glass).cuda(), 100.0, 2)
    d_gpu = periodic_delta(pos.cpu().numpy(), lagr, cfg["Box"])
    d_ref = periodic_delta(r["pos"], lagr, cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-5
    assert rel_rms(vel.cpu().numpy(), r["vel"]) < 1e-5
    assert np.array_equal(ids.cpu().numpy(), np.arange(1, len(lagr) + 1))


def test_run_host_matches_device(cuda):
    cfg = SMALL[1]
    r = oracle_run(key(cfg))
    g = gen_for(cfg)
    pos_d, vel_d = g.run(torch.from_numpy(r["lagr"]).cuda())
    torch.cuda.synchronize()
    pos_h, vel_h = g.run_host(r["lagr"])
    assert np.array_equal(pos_h, pos_d.cpu().numpy()) and np.array_equal(vel_h, vel_d.cpu().numpy())


def test_run_host_chunked_read_out(cuda):
    """2M particles: the host entry point reads out in chunks whose copies to
    the host overlap the next chunks; bit-identical to the device entry point."""
    cfg = make_cfg(128, 500.0, 21, 10.0, 8, "local_m8_L500_n128", 128)
    g = gen_for(cfg)
    rng = np.random.default_rng(4)
    lagr = rng.uniform(0, 500.0, (128 ** 3, 3)).astype(np.float32)
    pos_d, vel_d = g.run(torch.from_numpy(lagr).cuda())
    torch.cuda.synchronize()
    pos_h, vel_h = g.run_host(lagr)
    assert np.array_equal(pos_h, pos_d.cpu().numpy()) and np.array_equal(vel_h, vel_d.cpu().numpy())


def test_seed_changes_realisation(cuda):
    cfg = SMALL[0]
    g = gen_for(cfg)
    a = g.seedtable().cpu()
    g.set_seed(cfg["Seed"] + 1)
    b = g.seedtable().cpu()
    assert not torch.equal(a, b)


def test_error_codes_without_faults(cuda):
    from aarambam_gb300._lib import AAR_ERR_ARG, AAR_ERR_NMAX, AAR_ERR_OOM, AAR_ERR_TRANSFER, AarError
    from aarambam_gb300.ic import ICGenerator
    alpha, x0 = table("local_m8_L500_n128", 8)
    k, t = bbks()
    with pytest.raises(AarError) as e:
        ICGenerator(make_cfg(32, 500.0, 1, 10.0, 8, "x", Nmax=16), alpha, x0, k, t)
    assert e.value.code == AAR_ERR_NMAX
    with pytest.raises(AarError) as e:
        ICGenerator(make_cfg(48, 500.0, 1, 10.0, 8, "x", Nmax=128), alpha, x0, k, t)
    assert e.value.code == AAR_ERR_ARG
    kk = np.logspace(-3, 2, 100)
    with pytest.raises(AarError) as e:
        ICGenerator(make_cfg(32, 500.0, 1, 10.0, 8, "x", Nmax=128), alpha, x0, kk, np.ones_like(kk))
    assert e.value.code == AAR_ERR_TRANSFER
    with pytest.raises(AarError) as e:
        ICGenerator(make_cfg(64, 500.0, 1, 10.0, 8, "x", Nmax=128), alpha, x0, k, t, mem_limit_bytes=1 << 16)
    assert e.value.code == AAR_ERR_OOM
    bad = alpha.copy()
    bad[1, 1, 1] = np.nan
    with pytest.raises(AarError) as e:
        ICGenerator(make_cfg(32, 500.0, 1, 10.0, 8, "x", Nmax=128), bad, x0, k, t)
    assert e.value.code == AAR_ERR_ARG


@pytest.mark.parametrize("cfg", SMALL, ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_plain_fp64_form_vs_oracle(cuda, cfg):
    """cuFFT FP64 form, loop structure of the reference: agrees with the FP64
    oracle to FP64 rounding (FFT algorithms and table-evaluated powers differ)."""
    r = oracle_run(key(cfg))
    g = gen_for(cfg, precision="fp64")
    pos, vel = g.run(torch.from_numpy(r["lagr"]).cuda())
    d_gpu = periodic_delta(pos.cpu().numpy(), r["lagr"], cfg["Box"])
    d_ref = periodic_delta(r["pos"], r["lagr"], cfg["Box"])
    # positions are stored as float32 (main.c part_data): compare at that level
    assert rel_rms(d_gpu, d_ref) < 1e-6
    assert rel_rms(vel.cpu().numpy(), r["vel"]) < 1e-6
    assert g.launches > 10


@pytest.mark.parametrize("cfg", SMALL, ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_plain_fp64_regrouped_vs_oracle(cuda, cfg):
    """Regrouped plain FP64 form (M c2r + R r2c, counter-terms folded into
    alpha'): particles agree with the FP64 oracle at the float32 storage
    level, and its FP64 displacement fields and total potential agree with
    the oracle's to FP64 rounding (different summation order and no
    potential round trips)."""
    r = oracle_run(key(cfg))
    g = gen_for(cfg, precision="fp64_regrouped")
    pos, vel = g.run(torch.from_numpy(r["lagr"]).cuda())
    d_gpu = periodic_delta(pos.cpu().numpy(), r["lagr"], cfg["Box"])
    d_ref = periodic_delta(r["pos"], r["lagr"], cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-6
    assert rel_rms(vel.cpu().numpy(), r["vel"]) < 1e-6
    f = np.stack([g.field(i).cpu().numpy() for i in range(6)])
    assert f.dtype == np.float64
    assert rel_rms(f[:3], r["disp"][:3]) < 1e-9
    assert rel_rms(f[3:], r["disp"][3:]) < 1e-9
    tot = r["total"][..., 0] + 1j * r["total"][..., 1]
    assert rel_rms(g.spectrum().cpu().numpy(), tot) < 1e-9


@pytest.mark.parametrize("cfg", SMALL[:2], ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_plain_fp64_fields_vs_oracle(cuda, cfg):
    """FP64 field copies of the reference-structure plain form (what the
    precision comparisons at full size use as the FP64 reference)."""
    r = oracle_run(key(cfg))
    g = gen_for(cfg, precision="fp64")
    g.run(torch.from_numpy(r["lagr"]).cuda())
    f = np.stack([g.field(i).cpu().numpy() for i in range(6)])
    assert rel_rms(f[:3], r["disp"][:3]) < 1e-9
    assert rel_rms(f[3:], r["disp"][3:]) < 1e-9


def test_run_glass_host_sync_and_async(cuda):
    """Host-buffer glass entry points: a random glass tiled 8^3 times (2.1M
    particles, 16 read-out chunks) gives the device entry point's particles
    bit for bit; two asynchronous calls with different seeds in a row (the
    second computing while the first copies out) each deliver their own
    realisation."""
    cfg = make_cfg(128, 500.0, 21, 10.0, 8, "local_m8_L500_n128", 128)
    g = gen_for(cfg)
    rng = np.random.default_rng(5)
    glass = rng.uniform(0, 100.0, (4096, 3)).astype(np.float32)
    dglass = torch.from_numpy(glass).cuda()
    want = []
    for seed in (21, 22):
        g.set_seed(seed)
        want.append([t.cpu() for t in g.run_glass(dglass, 100.0, 8)])
    g.set_seed(21)
    pos, vel, ids = g.run_glass_host(glass, 100.0, 8)
    assert np.array_equal(pos, want[0][0].numpy()) and np.array_equal(vel, want[0][1].numpy())
    assert np.array_equal(ids, want[0][2].numpy())
    n = glass.shape[0] * 8 ** 3
    bufs = [(torch.empty((n, 3), dtype=torch.float32).pin_memory(), torch.empty((n, 3), dtype=torch.float32).pin_memory(),
             torch.empty((n,), dtype=torch.int32).pin_memory()) for _ in range(2)]
    for seed, b in zip((21, 22), bufs):
        g.set_seed(seed)
        g.run_glass_host(glass, 100.0, 8, out=b, wait=False)
    g.wait_host_copies()
    torch.cuda.synchronize()
    for b, w in zip(bufs, want):
        assert all(torch.equal(x, y) for x, y in zip(b, w))


@pytest.mark.parametrize("cfg", SMALL[:4], ids=lambda c: f"N{c['Nmesh']}_s{c['Seed']}")
def test_gaussian_spectrum_fp64_amplitude(cuda, cfg):
    """noise_fp64: the fused form's RNG-to-amplitude step in FP64 with the
    reference's formula, rounded to float at the end -- bit-identical to the
    plain FP64 form's Gaussian spectrum rounded to complex64, and within
    float rounding of the FP64 oracle per cell."""
    import ctypes as C
    g = gen_for(cfg, noise_fp64=True)
    g.stage("noise")
    got = g.spectrum()
    gp = gen_for(cfg, precision="fp64")
    N = cfg["Nmesh"]
    ref = torch.empty((N, N, N // 2 + 1), dtype=torch.complex128, device=cuda)
    rc = gp.L.aar_gaussian_spectrum_noalloc(gp.h, ref.data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    assert torch.equal(got, ref.to(torch.complex64))
    k, t = bbks()
    o = O.Oracle(cfg, k, t).gauss()
    o = o[..., 0] + 1j * o[..., 1]
    got = got.cpu().numpy()
    nz = o != 0
    assert np.array_equal(got != 0, nz)
    assert (np.abs(got[nz] - o[nz]) / np.abs(o[nz])).max() < 2e-7


def lattice_expected(gen, cfg, g, glass_box, tile):
    """Positions and velocities of the lattice particles read straight off
    the grid (FP64 from the plan's FP32 displacement fields after
    aar_stage_lpt): each particle (x, y, z) moves by its grid point's
    psi1 - 3/7 psi2 / N^3 (main.c:1486-1509), particles in read_glass.c's
    tiled order."""
    N, box = cfg["Nmesh"], cfg["Box"]
    gen.stage("noise")
    gen.stage("modal")
    gen.stage("lpt")
    f = [gen.field(i).double() for i in range(6)]
    s = gen.scalars
    i = torch.arange(N, dtype=torch.float64, device=f[0].device)
    gi, ti = torch.remainder(i, g), torch.div(i, g, rounding_mode="floor")
    gc = (gi * (glass_box / g)).float().double()
    bot = box / tile
    lp = (gc / glass_box * bot + ti * bot).float().double()
    n3 = float(np.float32(float(N) ** 3))
    d2 = [x / n3 for x in f[3:]]
    pos = [lp.view(-1, 1, 1) if a == 0 else lp.view(1, -1, 1) if a == 1 else lp.view(1, 1, -1) for a in range(3)]
    P = torch.stack([torch.remainder(pos[a] + f[a] - 3.0 / 7.0 * d2[a], box) for a in range(3)], -1)
    V = torch.stack([f[a] * s["vel_prefac"] - 3.0 / 7.0 * d2[a] * s["vel_prefac2"] for a in range(3)], -1)
    # grid point (x, y, z) -> particle ((ti tile + tj) tile + tk) g^3 + (gi g + gj) g + gk
    X = torch.arange(N, device=f[0].device)
    t, q = torch.div(X, g, rounding_mode="floor"), torch.remainder(X, g)
    tx, ty, tz = t.view(-1, 1, 1), t.view(1, -1, 1), t.view(1, 1, -1)
    qx, qy, qz = q.view(-1, 1, 1), q.view(1, -1, 1), q.view(1, 1, -1)
    idx = (((tx * tile + ty) * tile + tz) * g ** 3 + (qx * g + qy) * g + qz).reshape(-1)
    Pn = torch.empty((N ** 3, 3), dtype=torch.float64, device=f[0].device)
    Vn = torch.empty_like(Pn)
    Pn[idx] = P.reshape(-1, 3)
    Vn[idx] = V.reshape(-1, 3)
    return Pn, Vn


def close_periodic(a, b, box, atol):
    """Positions equal to atol, modulo the box (a particle at the edge may
    wrap on one side and not the other)."""
    d = (a.double() - b.double()).abs()
    return bool(torch.all(torch.minimum(d, box - d) <= atol))


# (N, g, Box): N / Box a power of two puts every lattice point exactly on the
# grid in the general read-out's FP32 coordinate too (bit-identical paths);
# Box 500 / 1000 leave it fractions of ~1e-7 there; Box 777.7 puts the
# lattice off the grid (the general read-out runs inside aar_run_lattice)
@pytest.mark.parametrize("N,g,box", [(16, 8, 256.0), (32, 16, 512.0), (64, 16, 1000.0), (128, 64, 1024.0),
                                     (256, 64, 500.0), (512, 64, 1000.0), (64, 16, 777.7)])
def test_run_lattice_matches_glass(cuda, N, g, box):
    """aar_run_lattice (the regular g^3 lattice glass tiled N/g times, no
    glass array) against the general glass read-out and against the grid
    values under the particles."""
    from aarambam_gb300 import gadget
    cfg = make_cfg(N, box, 31, 100.0, 10, "scalarI_m10_L500_n256", max(N, 256))
    gen = gen_for(cfg)
    tile = N // g
    glass = torch.from_numpy(gadget.lattice_glass(g, 100.0)).cuda()
    pos_g, vel_g, ids_g = gen.run_glass(glass, 100.0, tile)
    pos = torch.full_like(pos_g, float("nan"))
    vel = torch.full_like(vel_g, float("nan"))
    ids = torch.zeros(N ** 3, dtype=torch.int32, device=cuda)
    gen.run_lattice(g, 100.0, tile, pos, vel, ids)
    assert torch.equal(ids, ids_g)
    vtol = 1e-6 * float(vel_g.abs().max())
    exact = box == 777.7 or (N / box) in [2.0 ** -k for k in range(12)]
    if exact:
        assert torch.equal(pos, pos_g) and torch.equal(vel, vel_g)
    else:
        assert close_periodic(pos, pos_g, box, 1e-4)
        torch.testing.assert_close(vel, vel_g, rtol=1e-6, atol=vtol)
    if box != 777.7:  # the fused read-out: the grid value under each particle
        P, V = lattice_expected(gen, cfg, g, 100.0, tile)
        assert close_periodic(pos, P, box, 1e-4)
        torch.testing.assert_close(vel.double(), V, rtol=1e-6, atol=vtol)
    # and through the host-glass entry point (lattice detected on the host):
    # the same read-out, bit for bit with aar_run_lattice
    hp, hv, hi = gen.run_glass_host(gadget.lattice_glass(g, 100.0), 100.0, tile)
    assert np.array_equal(hp, pos.cpu().numpy()) and np.array_equal(hv, vel.cpu().numpy())
    assert np.array_equal(hi, ids_g.cpu().numpy())

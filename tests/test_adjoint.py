"""Hand-written adjoint of the fused chain (white noise -> NG potential ->
2LPT displacements): gradients with respect to the noise and the alpha table
against an FP64 reference gradient (torch autograd over an FP64 restatement
of the same chain) and against central finite differences of the FP32
forward.  At 32^3 the reference chain uses the plan's own per-cell factors,
which are themselves checked against the reference's formulas; the
differentiation configuration (256^3, Box 500, ScalarI mass 1, 10 modes, 10 %
mask) builds every factor of its FP64 reference from the formulas
(main.c:405-459, 580-637, 825-867, 1180-1368) with the oracle's transfer
function and scalars, independent of the plan."""
import ctypes as C
import time

import numpy as np
import pytest
import torch

from aarambam_gb300 import _lib
from aarambam_gb300.adjoint import FWD, GAUSS, HESS, ONE, PSI1, PSI2, Q, RHO, _Ops, displacement, white_noise
from aarambam_gb300.ic import ICGenerator
from tests.common import bbks, make_cfg, table

pytestmark = pytest.mark.gpu

TAB, M = "scalarI_m10_L500_n256", 10


def setup(cuda, N=32, fnl=300.0):
    cfg = make_cfg(N, 500.0, 11, fnl, M, TAB, 256)
    alpha, x0 = table(TAB, M)
    gen = ICGenerator(cfg, alpha, x0, *bbks())
    w = white_noise(N, 5, cuda)
    g = torch.Generator().manual_seed(9)
    mask = (torch.rand((N, N, N), generator=g) < 0.1).to(torch.float64).to(cuda)
    return gen, np.array(alpha), w, mask


def loss_of(disp, mask):
    return (mask * disp.double() ** 2).sum()


def plan_factors(gen):
    """The plan's per-cell factors (aar_adj_spectral), FP64 on the CPU."""
    ops = _Ops(gen)
    N = gen.N
    one = torch.ones((N, N, N // 2 + 1), dtype=torch.complex64, device=gen.device)

    def fac(op, comp):
        return ops.spec(op, comp, FWD, one).to(torch.complex128).cpu()
    return dict(g=fac(GAUSS, 0), q=[fac(Q, p) for p in range(M)], r=[fac(RHO, r) for r in range(M)],
                h=[fac(HESS, ab) for ab in range(6)], p1=[fac(PSI1, a) for a in range(3)],
                p2=[fac(PSI2, a) for a in range(3)])


def formula_factors(cfg, x0, dev):
    """The same factors restated in FP64 from the reference's formulas, with
    the oracle's transfer function and scalars (nothing from the plan):
    noise amplitude sqrt(Anorm k^ns) (2 pi/Box)^1.5 Beta / k^2 on the cells the
    draw writes (main.c:405-459), field filters q_n and radial parts rho_n
    (main.c:580-637, 825-860, kbar and the Legendre recurrence), Hessians
    -k_a k_b T/(D Beta) (main.c:1238-1277), psi1 i k_a T/(D Beta) smth and
    psi2 -i k_a / k^2 smth with smth = [sinc_x sinc_y sinc_z]^-2
    (main.c:1180-1216, 1311-1368).  Cube cut at Nsample / 2."""
    from oracle import oracle as O
    N, box, ns = cfg["Nmesh"], cfg["Box"], cfg["PrimordialIndex"]
    o = O.Oracle(cfg, *bbks())
    sc = o.scalars
    f64 = dict(dtype=torch.float64, device=dev)
    kF = 2 * np.pi / box
    idx = torch.arange(N, device=dev)
    sg = torch.where(idx < N // 2, idx, idx - N).to(torch.float64)
    kx, ky = sg[:, None, None], sg[None, :, None]
    kz = torch.arange(N // 2 + 1, **f64)[None, None, :]
    n2 = kx ** 2 + ky ** 2 + kz ** 2
    half = cfg["Nsample"] // 2
    keep = (kx.abs() <= half) & (ky.abs() <= half) & (kz <= half)
    on = keep & (n2 > 0)
    k = kF * torch.sqrt(n2)
    ks = torch.where(on, k, torch.ones_like(k))  # a safe k off the kept cells
    drawn = on & (idx[:, None, None] != N // 2) & (idx[None, :, None] != N // 2) & (kz < N // 2)
    amp = torch.sqrt(sc["Anorm"] * ks ** ns) * (2 * np.pi / box) ** 1.5 * sc["Beta"] / ks ** 2
    Fg = torch.where(drawn, amp, 0.0)
    s = (4 - ns) / 3
    kmin, kmax = kF, kF * cfg["Nmax"]
    kbar = -1 + 2 * (ks ** s - kmin ** s) / (kmax ** s - kmin ** s)
    P = [torch.ones_like(kbar), kbar]
    for l in range(2, M):
        P.append(((2 * l - 1) * kbar * P[l - 1] - (l - 1) * P[l - 2]) / l)
    n3 = float(N) ** 3
    q, r = [], []
    for n in range(M):
        if n <= 3:
            out = ks ** (s * (n - 3))
            inn = out * ks ** (4 - ns)
        else:
            d = P[n - 1] - float(x0[n - 1])
            out = d / ks ** 2
            inn = d * ks ** (2 - ns)
        q.append(torch.where(on, inn, 0.0))
        r.append(torch.where(on, cfg["Fnl"] / n3 * out, 0.0))
    # T(k) / (D Beta) per |k|^2 from the oracle's transfer function
    n2i = n2.to(torch.int64)
    un = torch.unique(n2i).cpu().numpy()
    T = np.array([O.lib().orc_transfer(C.byref(o.p), kF * np.sqrt(float(m))) for m in un])
    tab = torch.zeros(int(un.max()) + 1, **f64)
    tab[torch.from_numpy(un).to(dev)] = torch.from_numpy(T / sc["Dplus"] / sc["Beta"]).to(dev)
    twb = tab[n2i]
    ka = [kF * kx, kF * ky, kF * kz]
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    h = [-ka[a] * ka[b] * twb for a, b in pairs]

    def sinc(kv):
        x = kv * box / 2 / N
        return torch.where(x == 0, torch.ones_like(x), torch.sin(x) / torch.where(x == 0, torch.ones_like(x), x))
    smth = (1.0 / (sinc(ka[0]) * sinc(ka[1]) * sinc(ka[2]))) ** 2
    k2 = kF ** 2 * n2
    p1 = [1j * ka[a] * twb * smth for a in range(3)]
    p2 = [torch.where(n2 > 0, -1j * ka[a] / torch.where(n2 > 0, k2, torch.ones_like(k2)) * smth, 0.0) for a in range(3)]
    c = lambda x: torch.as_tensor(x).to(torch.complex128).expand(N, N, N // 2 + 1)  # noqa: E731
    return dict(g=c(Fg), q=[c(x) for x in q], r=[c(x) for x in r], h=[c(x) for x in h], p1=[c(x) for x in p1],
                p2=[c(x) for x in p2])


def reference_chain(gen, w, alpha, mask, F=None, dev="cpu"):
    """FP64 restatement (torch autograd) of the chain, with the factors F
    (default: the plan's own)."""
    F = plan_factors(gen) if F is None else F
    N = gen.N
    Fg, Fq, Fr, Fh, F1, F2 = F["g"], F["q"], F["r"], F["h"], F["p1"], F["p2"]
    n3 = float(N) ** 3
    c2r = lambda x: torch.fft.irfftn(x, s=(N, N, N)) * n3  # noqa: E731  (FFTW c2r, unnormalised)
    r2c = torch.fft.rfftn
    wd = w.detach().to(torch.complex128).to(dev).requires_grad_(True)
    ad = torch.tensor(alpha, dtype=torch.float64, device=dev, requires_grad=True)
    phig = Fg * wd
    f = [c2r(Fq[p] * phig) for p in range(M)]
    g = [torch.zeros((N, N, N), dtype=torch.float64, device=dev) for _ in range(M)]
    for p in range(M):
        for q in range(p, M):
            for r in range(q, M):
                g[r] = g[r] + ad[p, q, r] * f[p] * f[q]
    if alpha[0, 1, 2] != 0:  # counter-terms of main.c:1045-1050
        g[2] = g[2] + ad[1, 1, 1] * f[0] * f[1]
        g[1] = g[1] - ad[1, 1, 1] * f[0] * f[2]
    phi = phig + sum(Fr[r] * r2c(g[r]) for r in range(M))
    d = [c2r(Fh[ab] * phi) for ab in range(6)]
    S = d[0] * (d[3] + d[5]) + d[3] * d[5] - d[1] ** 2 - d[2] ** 2 - d[4] ** 2
    Sh = r2c(S)
    disp = torch.stack([c2r(F1[a] * phi) - (3.0 / 7.0) / n3 * c2r(F2[a] * Sh) for a in range(3)])
    L = (mask.to(dev) * disp ** 2).sum()
    L.backward()
    return disp.detach(), wd.grad, ad.grad


def rel(a, b):
    a = torch.as_tensor(a).detach().to(torch.complex128)
    b = torch.as_tensor(b).detach().to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def test_adjoint_matches_fp64_reference_gradient(cuda):
    gen, alpha, w, mask = setup(cuda)
    wt = w.clone().requires_grad_(True)
    at = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    disp = displacement(gen, wt, at)
    loss_of(disp, mask).backward()
    rdisp, rgw, rga = reference_chain(gen, w, alpha, mask)
    assert rel(disp.cpu(), rdisp) < 1e-5
    assert rel(wt.grad.cpu(), rgw) < 1e-4
    sorted_ = np.zeros((M, M, M), bool)
    for p in range(M):
        for q in range(p, M):
            sorted_[p, q, q:] = True
    ga, ra = at.grad.cpu().numpy(), rga.numpy()
    assert np.all(ga[~sorted_] == 0)
    assert rel(ga[sorted_], ra[sorted_]) < 1e-4


def test_adjoint_central_differences(cuda):
    gen, alpha, w, mask = setup(cuda)
    wt = w.clone().requires_grad_(True)
    at = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    loss_of(displacement(gen, wt, at), mask).backward()
    gw, ga = wt.grad.clone(), at.grad.clone()
    eps = 1e-3
    g = torch.Generator().manual_seed(3)
    # noise: a random direction of the size of the noise
    v = torch.complex(torch.randn(w.shape, generator=g), torch.randn(w.shape, generator=g)).to(cuda)
    v = v * (torch.linalg.vector_norm(w) / torch.linalg.vector_norm(v))
    with torch.no_grad():
        lp = loss_of(displacement(gen, w + eps * v, at), mask).item()
        lm = loss_of(displacement(gen, w - eps * v, at), mask).item()
    fd = (lp - lm) / (2 * eps)
    an = float((gw.real * v.real + gw.imag * v.imag).sum())
    assert abs(fd - an) <= 2e-3 * abs(an)
    # alpha: a random direction over the nonzero sorted entries
    u = np.zeros_like(alpha)
    nz = np.argwhere(alpha != 0)
    rng = np.random.default_rng(4)
    for p, q, r in nz:
        if p <= q <= r:
            u[p, q, r] = rng.standard_normal()
    u *= np.abs(alpha[alpha != 0]).mean() / np.abs(u[u != 0]).mean()
    with torch.no_grad():
        lp = loss_of(displacement(gen, w, at + eps * torch.from_numpy(u)), mask).item()
        lm = loss_of(displacement(gen, w, at - eps * torch.from_numpy(u)), mask).item()
    fd = (lp - lm) / (2 * eps)
    an = float((ga * torch.from_numpy(u)).sum())
    assert abs(fd - an) <= 2e-3 * abs(an)


def test_plan_factors_match_formulas(cuda):
    """The plan's per-cell factors (FP32) against their FP64 restatement from
    the reference's formulas (the factors the 256^3 reference gradient uses)."""
    gen, alpha, w, mask = setup(cuda)
    _, x0 = table(TAB, M)
    Fp = plan_factors(gen)
    Ff = formula_factors(gen.cfg, x0, "cpu")
    for key in ("g", "q", "r", "h", "p1", "p2"):
        a = Fp[key] if isinstance(Fp[key], list) else [Fp[key]]
        b = Ff[key] if isinstance(Ff[key], list) else [Ff[key]]
        for i, (x, y) in enumerate(zip(a, b)):
            assert rel(x, y) < 2e-6, (key, i)


def setup_256(cuda):
    """The differentiation configuration: Nmesh 256, Box 500, ScalarI mass 1,
    10 modes, FP32; unit-variance noise; a random mask of 10 % of the
    particles (lattice particles sit on grid points, so a mask over cells)."""
    return setup(cuda, N=256, fnl=100.0)


def test_adjoint_256_vs_formula_fp64_gradient(cuda):
    gen, alpha, w, mask = setup_256(cuda)
    _, x0 = table(TAB, M)
    wt = w.clone().requires_grad_(True)
    at = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    disp = displacement(gen, wt, at)  # first pass compiles and allocates
    loss_of(disp, mask).backward()
    wt.grad = None
    at.grad = None
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    t0 = time.perf_counter()
    disp = displacement(gen, wt, at)
    L = loss_of(disp, mask)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    peak = torch.cuda.max_memory_allocated() + gen.device_bytes
    print(f"adjoint 256^3 M={M}: forward {1e3 * (t1 - t0):.1f} ms, backward {1e3 * (t2 - t1):.1f} ms, "
          f"peak device memory {peak / 2**30:.2f} GiB (torch {torch.cuda.max_memory_allocated() / 2**30:.2f} "
          f"+ plan {gen.device_bytes / 2**30:.2f})")
    F = formula_factors(gen.cfg, x0, cuda)
    rdisp, rgw, rga = reference_chain(gen, w, alpha, mask, F=F, dev=cuda)
    assert rel(disp, rdisp) < 1e-5
    assert rel(wt.grad, rgw) < 1e-4
    sorted_ = np.zeros((M, M, M), bool)
    for p in range(M):
        for q in range(p, M):
            sorted_[p, q, q:] = True
    ga, ra = at.grad.cpu().numpy(), rga.cpu().numpy()
    assert np.all(ga[~sorted_] == 0)
    assert rel(ga[sorted_], ra[sorted_]) < 1e-4


def test_adjoint_256_central_differences(cuda):
    """Central differences (eps = 1e-3) of the FP32 forward at 256^3 along a
    random noise direction and a random direction over the nonzero sorted
    alpha entries."""
    gen, alpha, w, mask = setup_256(cuda)
    wt = w.clone().requires_grad_(True)
    at = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    loss_of(displacement(gen, wt, at), mask).backward()
    gw, ga = wt.grad.clone(), at.grad.clone()
    eps = 1e-3
    g = torch.Generator().manual_seed(3)
    v = torch.complex(torch.randn(w.shape, generator=g), torch.randn(w.shape, generator=g)).to(cuda)
    v = v * (torch.linalg.vector_norm(w) / torch.linalg.vector_norm(v))
    with torch.no_grad():
        lp = loss_of(displacement(gen, w + eps * v, at), mask).item()
        lm = loss_of(displacement(gen, w - eps * v, at), mask).item()
    fd = (lp - lm) / (2 * eps)
    an = float((gw.real * v.real + gw.imag * v.imag).sum())
    assert abs(fd - an) <= 2e-3 * abs(an)
    u = np.zeros_like(alpha)
    rng = np.random.default_rng(4)
    for p, q, r in np.argwhere(alpha != 0):
        if p <= q <= r:
            u[p, q, r] = rng.standard_normal()
    u *= np.abs(alpha[alpha != 0]).mean() / np.abs(u[u != 0]).mean()
    with torch.no_grad():
        lp = loss_of(displacement(gen, w, at + eps * torch.from_numpy(u)), mask).item()
        lm = loss_of(displacement(gen, w, at - eps * torch.from_numpy(u)), mask).item()
    fd = (lp - lm) / (2 * eps)
    an = float((ga * torch.from_numpy(u)).sum())
    assert abs(fd - an) <= 2e-3 * abs(an)

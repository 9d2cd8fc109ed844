"""Hand-written adjoint of the fused chain (white noise -> NG potential ->
2LPT displacements): gradients with respect to the noise and the alpha table
against an FP64 reference gradient (torch autograd over an FP64 restatement
of the same chain, with the plan's own per-cell factors) and against central
finite differences of the FP32 forward."""
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


def reference_chain(gen, w, alpha, mask):
    """FP64 restatement (torch, CPU) of the chain with the plan's factors."""
    ops = _Ops(gen)
    N = gen.N
    one = torch.ones((N, N, N // 2 + 1), dtype=torch.complex64, device=w.device)

    def fac(op, comp):
        return ops.spec(op, comp, FWD, one).to(torch.complex128).cpu()
    Fg = fac(GAUSS, 0)
    Fq = [fac(Q, p) for p in range(M)]
    Fr = [fac(RHO, r) for r in range(M)]
    Fh = [fac(HESS, ab) for ab in range(6)]
    F1 = [fac(PSI1, a) for a in range(3)]
    F2 = [fac(PSI2, a) for a in range(3)]
    n3 = float(N) ** 3
    c2r = lambda x: torch.fft.irfftn(x, s=(N, N, N)) * n3  # noqa: E731  (FFTW c2r, unnormalised)
    r2c = torch.fft.rfftn
    wd = w.detach().to(torch.complex128).cpu().requires_grad_(True)
    ad = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    phig = Fg * wd
    f = [c2r(Fq[p] * phig) for p in range(M)]
    g = [torch.zeros((N, N, N), dtype=torch.float64) for _ in range(M)]
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
    L = (mask.cpu() * disp ** 2).sum()
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

"""Differentiable fused path: white noise -> Gaussian potential -> modal
non-Gaussian potential -> ZA + 2LPT displacement field, as a
torch.autograd.Function with a hand-written adjoint.

`displacement(gen, w_hat, alpha)` returns the displacement field on the grid,
float32 [3, N, N, N]:

    disp_a = psi1_a - (3/7) psi2_a / N^3

with psi1 / psi2 the ZA and 2LPT fields exactly as the path reads them out
at the particles (Aarambam/LPT/Basis/main.c:1486-1507: Pos += dis - 3/7 dis2,
dis2 /= N^3).  Inputs:
  w_hat  complex64 [N, N, N/2+1]: the unit-variance noise whose scaled copy
         amp(k) w_hat is the Gaussian potential (the reference draws
         w = sqrt(-ln u2) e^{2 pi i u1}, main.c:396-459);
  alpha  float64 [M, M, M]: the coefficient table; entries with p <= q <= r
         are the ones the path reads (the reference symmetrises the
         AlphaTable rows, main.c:233-241), and the gradient is returned there.

The backward pass is the transpose of every step (aarambam_gb300/csrc/
adjoint.cu has the per-cell factors and the real-space products); it runs the
plan's own FFTs and recomputes the M filtered fields f_p and the six
Hessians from the saved spectra instead of storing them (memory: the noise,
the Gaussian and the total potential spectra are saved; the backward holds
about 2M + 12 fields at its peak).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check
from .ic import ICGenerator, _ptr

ONE, GAUSS, Q, RHO = _lib.AAR_ADJ_OP_ONE, _lib.AAR_ADJ_OP_GAUSS, _lib.AAR_ADJ_OP_Q, _lib.AAR_ADJ_OP_RHO
HESS, PSI1, PSI2 = _lib.AAR_ADJ_OP_HESS, _lib.AAR_ADJ_OP_PSI1, _lib.AAR_ADJ_OP_PSI2
FWD, CT_W, CT_INV_W, CT = 0, 1, 2, 3  # factor modes: F, conj(F) w, conj(F)/w, conj(F)


class _Ops:
    """Thin wrappers over the plan's C-ABI building blocks."""

    def __init__(self, gen: ICGenerator):
        self.g = gen
        self.L = gen.L
        self.N = gen.N

    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.g.device).cuda_stream)

    def spec(self, op, comp, mode, x, out=None):
        acc = out is not None
        if out is None:
            out = torch.empty_like(x)
        check(self.L, self.g.h, self.L.aar_adj_spectral(self.g.h, op, comp, mode, _ptr(x), _ptr(out), int(acc),
                                                        self.stream()))
        return out

    def c2r(self, x):
        return self.g.c2r(x)

    def r2c(self, x):
        return self.g.r2c(x)

    def set_spectrum(self, x):
        check(self.L, self.g.h, self.L.aar_set_spectrum(self.g.h, _ptr(x), self.stream()))

    def source_adj(self, d, gS):
        out = torch.empty_like(d)
        check(self.L, self.g.h, self.L.aar_adj_source(self.g.h, _ptr(d), _ptr(gS), _ptr(out), self.stream()))
        return out

    def products_adj(self, f, gg):
        M = f.shape[0]
        gf = torch.empty_like(f)
        ga = torch.zeros((M, M, M), dtype=torch.float64, device=f.device)
        check(self.L, self.g.h, self.L.aar_adj_products(self.g.h, _ptr(f), _ptr(gg), _ptr(gf), _ptr(ga),
                                                        self.stream()))
        return gf, ga


class _Displacement(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w_hat, alpha, gen):
        ops = _Ops(gen)
        N = gen.N
        ctx.w_dtype = w_hat.dtype
        w_hat = w_hat.to(torch.complex64).contiguous()
        gen.set_tables(alpha.detach().double().cpu().numpy())
        phig = ops.spec(GAUSS, 0, FWD, w_hat)
        ops.set_spectrum(phig)
        gen.stage("modal")
        phi = gen.spectrum()
        gen.stage("lpt")
        f = [gen.field(i) for i in range(6)]
        disp = torch.stack(f[:3]) - (3.0 / 7.0) / float(N) ** 3 * torch.stack(f[3:])
        ctx.gen = gen
        ctx.save_for_backward(phig, phi)
        ctx.alpha_dtype, ctx.alpha_device = alpha.dtype, alpha.device
        return disp

    @staticmethod
    def backward(ctx, gdisp):
        gen = ctx.gen
        ops = _Ops(gen)
        phig, phi = ctx.saved_tensors
        N, M = gen.N, gen.n_modes
        gdisp = gdisp.to(torch.float32).contiguous()
        # ZA and 2LPT read-outs: psi1 and -(3/7)/N^3 psi2
        gphi = torch.zeros_like(phi)
        gsrc = torch.zeros_like(phi)
        c2 = -(3.0 / 7.0) / float(N) ** 3
        for a in range(3):
            ops.spec(PSI1, a, CT_W, ops.r2c(gdisp[a].contiguous()), out=gphi)
            ops.spec(PSI2, a, CT_W, ops.r2c((c2 * gdisp[a]).contiguous()), out=gsrc)
        gS = ops.c2r(ops.spec(ONE, 0, CT_INV_W, gsrc))
        del gsrc
        # source S(d) with the Hessians recomputed from phi
        d = torch.stack([ops.c2r(ops.spec(HESS, ab, FWD, phi)) for ab in range(6)])
        gd = ops.source_adj(d, gS)
        del d, gS
        for ab in range(6):
            ops.spec(HESS, ab, CT_W, ops.r2c(gd[ab].contiguous()), out=gphi)
        del gd
        # modal part: phi = phig + sum_r rho_r r2c(g_r), g_r = sum alpha' f_p f_q
        gg = torch.stack([ops.c2r(ops.spec(RHO, r, CT_INV_W, gphi)) for r in range(M)])
        f = torch.stack([ops.c2r(ops.spec(Q, p, FWD, phig)) for p in range(M)])
        gf, galpha = ops.products_adj(f, gg)
        del f, gg
        gphig = gphi
        for p in range(M):
            ops.spec(Q, p, CT_W, ops.r2c(gf[p].contiguous()), out=gphig)
        gw = ops.spec(GAUSS, 0, CT, gphig)
        return gw.to(ctx.w_dtype), galpha.to(device=ctx.alpha_device, dtype=ctx.alpha_dtype), None


def displacement(gen: ICGenerator, w_hat: torch.Tensor, alpha: torch.Tensor) -> torch.Tensor:
    """Differentiable displacement field float32 [3, N, N, N] (see the module
    docstring); gradients flow to w_hat and alpha."""
    return _Displacement.apply(w_hat, alpha, gen)


def white_noise(N: int, seed: int, device) -> torch.Tensor:
    """Unit-variance complex noise of the shape the path takes (torch's
    generator; for tests and examples)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    u1 = torch.rand((N, N, N // 2 + 1), generator=g, dtype=torch.float64)
    u2 = 1.0 - torch.rand((N, N, N // 2 + 1), generator=g, dtype=torch.float64)
    w = torch.sqrt(-torch.log(u2)) * torch.exp(2j * np.pi * u1)
    return w.to(torch.complex64).to(device)

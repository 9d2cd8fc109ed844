"""The split-digit covariance scheme of csrc/gram_tc.cu, emulated on the CPU:
the digit cut and its bf16 tiles in the tcgen05 no-swizzle K-major layout
(written with the kernel's index arithmetic, read back as the shared-memory
descriptor addresses them), the seven level accumulators (levels 0-5 checked
exact in FP32 over every 128-point group, 6 and 7 rounded to FP32 after every
16-point step) and the int64 fixed-point read-out, against the FP64 oracle
covariance pinned to the reference's compiled kernels."""
import os

import numpy as np

from oracle import decomp as D
from tests.common import GOLDEN

TM, TN, TK, GROUP, NDIG = 128, 64, 16, 8, 8
LBO, SBO = 128, 256  # descriptor byte offsets: next core matrix along K, next 8-row group


def digits(x, e):
    """d_s 2^(-8 s), s = 0..7, of rint(x 2^(62 - e)) (balanced 8-bit digits)."""
    v = np.rint(np.ldexp(x, 62 - e)).astype(np.int64)
    d = np.zeros(x.shape + (NDIG,))
    for s in range(NDIG - 1, 0, -1):
        lo = ((v + 128) & 255) - 128
        d[..., s] = np.ldexp(lo.astype(np.float64), -8 * s)
        v = (v - lo) >> 8
    d[..., 0] = v
    assert np.abs(d[..., 0]).max() <= 64 and np.abs(np.ldexp(d[..., 1:], 8 * np.arange(1, NDIG))).max() <= 128
    return d


def covariance_split_digits(w, tidx, midx, mev):
    Q = D.mode_bispectra(tidx, midx, mev)
    nm, npts = Q.shape
    npad = -(-npts // (TK * GROUP)) * TK * GROUP
    nch = npad // TK
    ntA, ntB = -(-nm // TM), -(-nm // TN)
    rowsA, rowsB = ntA * TM, ntB * TN
    Qp = np.zeros((rowsA, npad))
    Qp[:nm, :npts] = Q
    wp = np.zeros(npad)
    wp[:npts] = w
    A = Qp * wp[None, :]
    mA, mB = np.abs(A).max(1), np.abs(Qp).max(1)
    eA = np.where(mA > 0, np.frexp(mA)[1], 0)
    eB = np.where(mB > 0, np.frexp(mB)[1], 0)
    # k_tetra_digits: 16-byte units (8 points of one row) per (tile, chunk, digit)
    u = np.arange(256)
    r, kseg = (u >> 4) * 8 + (u & 7), (u >> 3) & 1
    adig = np.zeros((ntA * nch * NDIG * 256, 8))
    bdig = np.zeros((ntB * nch * NDIG * 128, 8))
    c = np.arange(nch)[:, None, None]
    t = c * TK + kseg[None, :, None] * 8 + np.arange(8)[None, None, :]  # [chunk][unit][point]
    for I in range(ntA):
        n = I * TM + r
        dA = digits(A[n[None, :, None], t], eA[n][None, :, None])  # [chunk][unit][point][digit]
        dB = digits(Qp[n[None, :, None], t], eB[n][None, :, None])
        blk = I * nch + np.arange(nch)
        for s in range(NDIG):
            adig[((blk[:, None] * NDIG + s) * 256 + u[None, :]).ravel()] = dA[..., s].reshape(-1, 8)
        ok = n < rowsB
        J, rb = n // TN, n % TN
        ub = (rb >> 3) * 16 + kseg * 8 + (rb & 7)
        for s in range(NDIG):
            idx = ((J[None, :] * nch + np.arange(nch)[:, None]) * NDIG + s) * 128 + ub[None, :]
            bdig[idx[:, ok].ravel()] = dB[..., s][:, ok].reshape(-1, 8)
    aflat, bflat = adig.ravel(), bdig.ravel()

    def tile(flat, blocks, rows):  # [chunk][row][k] through the descriptor's addressing
        i, k = np.arange(rows)[:, None], np.arange(TK)[None, :]
        off = (i // 8) * SBO + (k // 8) * LBO + (i % 8) * 16 + (k % 8) * 2
        return flat[(blocks[:, None, None] + off[None]) // 2]

    qq = np.zeros((nm, nm))
    for I in range(ntA):
        for J in range(2 * I, ntB):
            a = [tile(aflat, ((I * nch + np.arange(nch)) * NDIG + s) * TM * TK * 2, TM) for s in range(NDIG)]
            b = [tile(bflat, ((J * nch + np.arange(nch)) * NDIG + s) * TN * TK * 2, TN) for s in range(NDIG)]
            # per chunk and level: sum over the level's digit pairs, exact in FP64
            lev = [sum(np.einsum("cik,cjk->cij", a[s], b[L - s]) for s in range(L + 1)) for L in range(NDIG)]
            hi = np.zeros((TM, TN), np.int64)
            lo = np.zeros((TM, TN), np.int64)
            for g in range(0, nch, GROUP):
                ints = []
                for L in range(6):
                    acc = lev[L][g:g + GROUP].sum(0)
                    x = np.ldexp(acc, 8 * L)
                    assert np.all(np.abs(x) < 2 ** 24) and np.all(x == np.rint(x))  # exact in FP32
                    ints.append(x.astype(np.int64))
                acc67 = np.zeros((TM, TN), np.float32)
                for cc in range(g, g + GROUP):
                    acc67 = (acc67 + lev[6][cc] + lev[7][cc]).astype(np.float32)
                i67 = np.rint(np.ldexp(acc67.astype(np.float64), 56)).astype(np.int64)
                hi += ints[0] * 65536 + ints[1] * 256 + ints[2]
                lo += ints[3] * 4294967296 + ints[4] * 16777216 + ints[5] * 65536 + i67
                hi += lo >> 40
                lo &= 0xFFFFFFFFFF
            n = I * TM + np.arange(TM)[:, None]
            m = J * TN + np.arange(TN)[None, :]
            keep = (n < nm) & (m < nm) & (n <= m)
            sc = eA[np.minimum(n, rowsA - 1)] + eB[np.minimum(m, rowsB - 1)]
            v = np.ldexp(hi.astype(np.float64), sc - 28) + np.ldexp(lo.astype(np.float64), sc - 68)
            nn, mm = np.nonzero(keep)
            qq[I * TM + nn, J * TN + mm] = v[nn, mm]
            qq[J * TN + mm, I * TM + nn] = v[nn, mm]
    return qq


def test_split_digit_covariance_matches_oracle():
    z = np.load(os.path.join(GOLDEN, "decomp", "small_m6_k24.npz"))
    args = (z["tetrapyd_grid_weights"], z["tetrapyd_indices"], z["mode_indices"], z["mode_evals"])
    got = covariance_split_digits(*args)
    want = D.covariance(*args)
    assert np.array_equal(got, got.T)
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()
    assert np.abs(got - z["QQ"]).max() <= 1e-14 * np.abs(z["QQ"]).max()


def test_split_digit_covariance_several_tiles():
    """165 modes (two A tiles of 128 rows, three B tiles of 64) on 5950
    points (47 groups): every tile pair of the upper triangle."""
    from aarambam_gb300 import basis as B
    kF = 2 * np.pi / 1000.0
    b = B.Basis(k_min=kF, k_max=kF * 512, parameter_n_scalar=0.965, mode_p_max=9, k_grid_size=40, host_only=True)
    args = (b.tetrapyd_grid_weights, b.tetrapyd_indices, b.mode_indices, b.mode_function_evaluations)
    got = covariance_split_digits(*args)
    want = D.covariance(*args)
    assert got.shape == (165, 165) and np.array_equal(got, got.T)
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()


# ---- host side of csrc/gram_tc.cu and the stored-mode entry points (no device work) ----
def _lib_handle():
    from aarambam_gb300 import _lib
    return _lib, _lib.load(build_if_missing=True)


def test_stored_mode_stride_and_scratch_sizes():
    """Q rows padded to whole 128-point groups; the covariance scratch holds at
    least the bf16 digit tiles (8 digits of 128-row A tiles and 64-row B
    tiles per 16-point chunk) and the stateless form adds the Q it makes."""
    _, L = _lib_handle()
    for npts, ld in [(1, 128), (128, 128), (129, 256), (289750, 289792)]:
        assert L.aar_tetra_modes_ld(npts) == ld
    assert L.aar_tetra_modes_ld(0) == 0
    nm, npts = 1540, 289750
    nch = 289792 // 16
    digits = (13 * nch * 8 * 4096) + (25 * nch * 8 * 2048)
    modes = L.aar_modes_covariance_scratch_bytes(npts, nm)
    assert digits < modes < digits * 1.05
    assert L.aar_tetra_covariance_scratch_bytes(npts, nm) >= modes + nm * 289792 * 8
    assert L.aar_modes_covariance_scratch_bytes(0, nm) == 0 and L.aar_modes_covariance_scratch_bytes(npts, 0) == 0


def test_stored_mode_argument_errors():
    """Argument checks that return before any device work: a Q stride other
    than aar_tetra_modes_ld, a Q base that is not 16-byte aligned, too little
    scratch, null pointers."""
    import ctypes as C
    _lib, L = _lib_handle()
    p = C.c_void_p(4096)  # never dereferenced: every call below fails its checks first
    npts, nm = 1000, 56
    ld = L.aar_tetra_modes_ld(npts)
    need = L.aar_modes_covariance_scratch_bytes(npts, nm)
    bad = [
        L.aar_modes_covariance(p, p, ld + 128, p, npts, nm, p, C.c_size_t(need), None),
        L.aar_modes_covariance(p, C.c_void_p(4104), ld, p, npts, nm, p, C.c_size_t(need), None),
        L.aar_modes_covariance(p, p, ld, p, npts, nm, p, C.c_size_t(need - 1), None),
        L.aar_modes_covariance(None, p, ld, p, npts, nm, p, C.c_size_t(need), None),
        L.aar_modes_project(p, p, 1, p, None, ld, npts, nm, None),
        L.aar_modes_project(p, p, 1, p, p, npts - 1, npts, nm, None),
        L.aar_modes_residual(p, p, None, None, 3, p, ld, npts, None),
        L.aar_tetra_modes(p, npts - 1, p, p, p, npts, p, p, p, nm, p, 6, 24, None),
    ]
    assert all(rc == _lib.AAR_ERR_ARG for rc in bad), bad

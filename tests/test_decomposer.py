"""Modal decomposition (the Decomposer): host parts on the CPU, the FP64 GPU
kernels against the oracle pinned to the reference's own compiled kernels
(tests/golden/decomp/small_m6_k24.npz), and whole decompositions against the
coefficient tables the reference Decomposer wrote (tests/golden/tables)."""
import json
import os

import numpy as np
import pytest

from aarambam_gb300 import basis as B
from aarambam_gb300 import models, utils
from oracle import decomp as D
from tests.common import GOLDEN

SMALL = os.path.join(GOLDEN, "decomp", "small_m6_k24.npz")


def small_basis(**kw):
    kF = 2 * np.pi / 500.0
    return B.Basis(k_min=kF, k_max=kF * 128, parameter_n_scalar=0.965, mode_p_max=6, k_grid_size=24, **kw)


def meta(name):
    with open(os.path.join(GOLDEN, "tables", name, "meta.json")) as f:
        return json.load(f)


def golden_table(name):
    return np.loadtxt(os.path.join(GOLDEN, "tables", name, "AlphaTable.dat"))


# ------------------------------------------------------------ CPU
def test_oracle_matches_reference_kernels():
    z = np.load(SMALL)
    args = (z["tetrapyd_grid_weights"], z["tetrapyd_indices"], z["mode_indices"], z["mode_evals"])
    qq = D.covariance(*args)
    assert np.abs(qq - z["QQ"]).max() <= 1e-13 * np.abs(z["QQ"]).max()
    qs = D.project(z["S"], *args)
    assert np.abs(qs - z["QS"]).max() <= 1e-13 * np.abs(z["QS"]).max()
    norms = np.sqrt(np.diag(z["QQ"]))
    qqt = z["QQ"] / norms[:, None] / norms[None, :]
    got = np.concatenate([[D.cond(i, m, qqt) for i in np.where(~m)[0]] for m in z["masks"]])
    assert np.allclose(got, z["conds"], rtol=1e-10)


def test_host_grids_match_reference():
    z = np.load(SMALL)
    b = small_basis(host_only=True)
    assert np.array_equal(b.k_grid, z["k_grid"]) and np.array_equal(b.k_weights, z["k_weights"])
    assert np.array_equal(b.tetrapyd_indices, z["tetrapyd_indices"])
    assert np.array_equal(b.tetrapyd_grid_weights, z["tetrapyd_grid_weights"])
    assert np.array_equal(b.mode_indices, z["mode_indices"])
    assert np.allclose(b.mode_function_evaluations, z["mode_evals"], rtol=1e-14, atol=0)


def test_scalarI_tetrapyd_order_matches_fixture():
    z = np.load(os.path.join(GOLDEN, "decomp", "scalarI_m10_L500_n256_S.npz"))
    kF = 2 * np.pi / 500.0
    b = B.Basis(k_min=kF, k_max=kF * 256, parameter_n_scalar=0.965, mode_p_max=10, k_grid_size=150, host_only=True)
    assert np.array_equal(b.tetrapyd_indices, z["tetrapyd_indices"].astype(np.int64))


@pytest.mark.parametrize("name", ["local_m8_L500_n128", "scalarI_m10_L500_n256", "scalarI_m20_L1000_n1024"])
def test_ai_table_matches_reference(name):
    m = meta(name)
    dec = B.BasicBasisDecompose(m["N_modes"], m["n_s"], m["Lbox"], m["Nmax"], m["ModeTol"], m["MaxModeCount"])
    got = dec.generate_Ai()["AiTable"]
    want = np.loadtxt(os.path.join(GOLDEN, "tables", name, "AiTable.dat"))
    assert np.allclose(got, want, rtol=1e-15, atol=1e-15)


def test_models_are_plugins():
    C = type("C", (models.Local, B.BasicBasisDecompose), {})
    inst = C(N_modes=8, n_s=0.965, Lbox=500.0, Nmax=128, ModeTol=1e-4, MaxModeCount=150)
    k = np.array([0.05, 0.1])
    # local template in the equilateral limit: S = (k^2 k^(2 (n_s - 2))) k^6 / k^6 = k^(2 n_s - 2)
    assert np.allclose(inst.shape_function(k, k, k), k ** (2 * 0.965 - 2))
    R = type("R", (models.LogResonance, B.BasicBasisDecompose), {})
    r = R(N_modes=8, n_s=0.965, Lbox=500.0, Nmax=128, ModeTol=1e-4, MaxModeCount=150, w_res=10.0, phi=0.0)
    assert np.isfinite(r.shape_function(k, k, 2 * k)).all()


# ------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_covariance_and_projection_vs_oracle(cuda):
    z = np.load(SMALL)
    b = small_basis(verbose=False)
    qq = b.mode_bispectra_covariance
    assert np.abs(qq - z["QQ"]).max() <= 1e-13 * np.abs(z["QQ"]).max()
    assert np.array_equal(qq, qq.T)
    qs = b.compute_QS_C(z["S"])
    assert np.abs(qs - z["QS"]).max() <= 1e-13 * np.abs(z["QS"]).max()


@pytest.mark.gpu
def test_covariance_tiles_and_slices(cuda):
    # several 128 x 64 tiles (M = 12: 364 modes) over several point ranges
    kF = 2 * np.pi / 1000.0
    b = B.Basis(k_min=kF, k_max=kF * 512, parameter_n_scalar=0.965, mode_p_max=12, k_grid_size=96, verbose=False)
    args = (b.tetrapyd_grid_weights, b.tetrapyd_indices, b.mode_indices, b.mode_function_evaluations)
    assert b.tetrapyd_grid_size > 65536
    want = D.covariance(*args)
    assert np.abs(b.mode_bispectra_covariance - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
@pytest.mark.parametrize("M,kgrid", [(1, 24), (2, 24), (30, 40)])
def test_covariance_edge_shapes_vs_oracle(cuda, M, kgrid):
    """The tensor-core covariance at the edges of its tiling: 1 and 4 modes
    (one 128 x 64 tile, nearly every row padding) and 30 modes (4960 3D
    modes: 39 x 78 tiles, 1560 tile pairs), against the oracle; and the
    projection at 4960 modes (its 32-warp block cap) against it too."""
    kF = 2 * np.pi / 1000.0
    b = B.Basis(k_min=kF, k_max=kF * 256, parameter_n_scalar=0.965, mode_p_max=M, k_grid_size=kgrid, verbose=False)
    args = (b.tetrapyd_grid_weights, b.tetrapyd_indices, b.mode_indices, b.mode_function_evaluations)
    want = D.covariance(*args)
    got = b.mode_bispectra_covariance
    assert got.shape == want.shape == (M * (M + 1) * (M + 2) // 6,) * 2
    assert np.array_equal(got, got.T)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    S = np.random.default_rng(M).standard_normal((1, b.tetrapyd_grid_size))
    qs, want_qs = b.compute_QS_C(S), D.project(S, *args)
    assert np.abs(qs - want_qs).max() <= 1e-13 * np.abs(want_qs).max()


@pytest.mark.gpu
def test_stored_modes_match_stateless_entry_points(cuda):
    """The stored-mode entry points the Basis uses (aar_modes_*, reading
    Q[n][t] made once by aar_tetra_modes) against the stateless ones
    (aar_tetra_*, evaluating Q_n(t) on the fly): the same terms in the same
    order, so the covariance, projections and residual agree bit for bit."""
    import ctypes as C

    import torch
    from aarambam_gb300 import _lib
    kF = 2 * np.pi / 1000.0
    b = B.Basis(k_min=kF, k_max=kF * 512, parameter_n_scalar=0.965, mode_p_max=12, k_grid_size=96, verbose=False)
    L = _lib.load()
    nm, npts = b.mode_indices.shape[1], b.tetrapyd_grid_size
    nbytes = L.aar_tetra_covariance_scratch_bytes(npts, nm)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    qq = torch.empty((nm, nm), dtype=torch.float64, device="cuda")
    b._call("aar_tetra_covariance", B._ptr(qq), *b._tetra_args(), B._ptr(scratch), C.c_size_t(nbytes), b._stream())
    assert np.array_equal(qq.cpu().numpy(), b.mode_bispectra_covariance)
    rng = np.random.default_rng(5)
    X = torch.from_numpy(rng.standard_normal((2, npts))).cuda()
    out = torch.empty((2, nm), dtype=torch.float64, device="cuda")
    b._call("aar_tetra_QS", B._ptr(out), B._ptr(X), 2, *b._tetra_args(), b._stream())
    assert np.array_equal(out.cpu().numpy(), b._project_dev(X).cpu().numpy())
    sel, coef = np.array([0, 7, 100, nm - 1]), rng.standard_normal(4)
    S = X[:1].contiguous()
    R = torch.empty_like(S)
    sel_d = torch.from_numpy(sel.astype(np.int32)).cuda()
    coef_d = torch.from_numpy(coef).cuda()
    b._call("aar_tetra_residual", B._ptr(R), B._ptr(S), B._ptr(sel_d), B._ptr(coef_d), 4, *b._tetra_args(),
            b._stream())
    assert np.array_equal(R.cpu().numpy(), b._residual_dev(S, sel, coef).cpu().numpy())


@pytest.mark.gpu
def test_residual_vs_oracle(cuda):
    import torch
    z = np.load(SMALL)
    b = small_basis(verbose=False)
    sel = np.array([1, 5, 17, 40, 55])
    coef = np.array([0.5, -1.25, 2.0, 1e-3, -0.75])
    S = torch.from_numpy(np.ascontiguousarray(z["S"][:1])).cuda()
    got = b._residual_dev(S, sel, coef).cpu().numpy()[0]
    want = D.residual(z["S"][0], sel, coef, z["tetrapyd_indices"], z["mode_indices"], z["mode_evals"])
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


@pytest.mark.gpu
def test_bordered_cond_vs_reference(cuda):
    import torch
    z = np.load(SMALL)
    b = small_basis(verbose=False)
    norms = np.sqrt(np.diag(z["QQ"]))
    qqt = z["QQ"] / norms[:, None] / norms[None, :]
    b._qq_tilde = qqt
    dev = torch.from_numpy(qqt).cuda()
    got = np.concatenate([b._candidate_conds(dev, m)[1] for m in z["masks"]])
    assert np.allclose(got, z["conds"], rtol=1e-7)


@pytest.mark.gpu
def test_bordered_cond_ill_conditioned(cuda):
    """Random PSD Gram matrices with condition numbers up to ~1e8 against
    np.linalg.cond of every bordered block."""
    import torch
    rng = np.random.default_rng(3)
    n = 60
    X = rng.standard_normal((n, 400)) * np.logspace(0, -4, n)[:, None]
    X[7] = X[3] + 1e-4 * X[7]  # a nearly dependent pair
    G = X @ X.T
    d = np.sqrt(np.diag(G))
    G = G / d[:, None] / d[None, :]
    b = small_basis(verbose=False)
    b._qq_tilde = G
    msk = np.zeros(n, dtype=bool)
    msk[:25] = True
    msk[7] = False
    cond_here, got = b._candidate_conds(torch.from_numpy(G).cuda(), msk)
    want = np.array([D.cond(i, msk, G) for i in np.where(~msk)[0]])
    assert abs(cond_here / np.linalg.cond(G[np.ix_(msk, msk)]) - 1) < 1e-6
    assert np.allclose(got, want, rtol=1e-6)
    assert want.max() > 1e6


@pytest.mark.gpu
def test_decomposer_local_matches_reference_table(cuda, tmp_path):
    name = "local_m8_L500_n128"
    m = meta(name)
    dec = utils.Decomposer(m["N_modes"], m["n_s"], m["Lbox"], m["Nmax"], m["ModeTol"], m["MaxModeCount"])
    out = dec.go(models.Local, B.BasicBasisDecompose, outdir=str(tmp_path), verbose=False)
    got = np.loadtxt(os.path.join(str(tmp_path), "AlphaTable.dat"))
    want = golden_table(name)
    assert np.array_equal(got[:, :3], want[:, :3])
    assert np.array_equal(got[:, 3] != 0, want[:, 3] != 0)
    # the template is one mode, (1, 1, 1), to 1e-10: that coefficient to
    # 1e-8, the other two are conjugate-gradient noise at the 1e-10 level in
    # both runs
    scale = np.abs(want[:, 3]).max()
    assert np.abs(got[:, 3] - want[:, 3]).max() <= 1e-8 * scale
    assert out["AlphaTable"].shape == want.shape


class _TabulatedScalarI:
    """The reference's ScalarI shape, tabulated on the k_grid_size 150
    tetrapyd (tests/golden/decomp/scalarI_m10_L500_n256_S.npz); other
    arguments (the diagnostic triangles) get zeros."""
    S = None

    def shape_function(self, k1, k2, k3):
        if np.shape(k1) == self.S.shape:
            return self.S.copy()
        return np.zeros_like(k1)


@pytest.mark.gpu
def test_decomposer_scalarI_matches_reference_table(cuda, tmp_path):
    """ScalarI, 10 modes: the matching pursuit picks the reference's modes in
    its first ~100 steps; beyond them the selected blocks have condition
    numbers above 1e7 and the capped conjugate-gradient solves (1000
    iterations, cmbbest.pyx:429) make each pick depend on rounding, so a
    restatement with any other summation order (the same numpy loop on the
    same CPU included) ends with a few different modes.  The expansion's
    quality is then what matches: the same number of modes and the shape
    correlation within 2e-5 of the reference table's."""
    name = "scalarI_m10_L500_n256"
    m = meta(name)
    _TabulatedScalarI.S = np.load(os.path.join(GOLDEN, "decomp", "scalarI_m10_L500_n256_S.npz"))["S"]
    dec = utils.Decomposer(m["N_modes"], m["n_s"], m["Lbox"], m["Nmax"], m["ModeTol"], m["MaxModeCount"])
    C = type("C", (_TabulatedScalarI, B.BasicBasisDecompose), {})
    inst = C(**dec.args, verbose=False)
    out = inst.go()
    got = out["AlphaTable"][:, 3]
    want = golden_table(name)[:, 3]
    ref_set = set(np.where(want != 0)[0])
    picks = [row[3] for row in inst.basis.omp_log]
    first_out = next((i for i, p in enumerate(picks) if p not in ref_set), len(picks))
    print("first pick outside the reference's modes:", first_out + 1, "of", len(picks))
    assert first_out >= 80
    assert np.count_nonzero(got) == np.count_nonzero(want)
    b = inst.basis
    S = _TabulatedScalarI.S
    QQ, QS = b.mode_bispectra_covariance, b.compute_QS_C(S)[0]
    SS = np.sum(S * S * b.tetrapyd_grid_weights)

    def corr(a):
        return (a @ QS) / np.sqrt(SS * (a @ QQ @ a))
    c_ref, c_got = corr(want), corr(got)
    print("correlation: reference table", c_ref, "this run", c_got)
    assert abs(c_ref - 0.9998542847) < 1e-8  # the reference table under this basis (CPU oracle: 0.99985428472)
    assert abs(c_got - c_ref) < 2e-5


@pytest.mark.gpu
def test_decomposer_logresonance_m20_matches_reference_table(cuda, tmp_path):
    """The resonant template of the 1536^3 case (LogResonance w_res = 10,
    20 modes, Lbox 2000, Nmax 1536): the pursuit runs its 129 steps to
    MaxModeCount and ends on the reference's 132 modes with the reference's
    coefficients."""
    name = "logres_w10_m20_L2000_n1536"
    m = meta(name)
    dec = utils.Decomposer(m["N_modes"], m["n_s"], m["Lbox"], m["Nmax"], m["ModeTol"], m["MaxModeCount"])
    dec.go(models.LogResonance, B.BasicBasisDecompose, outdir=str(tmp_path), verbose=False, **m["model_kwargs"])
    got = np.loadtxt(os.path.join(str(tmp_path), "AlphaTable.dat"))
    want = golden_table(name)
    assert np.array_equal(got[:, :3], want[:, :3])
    assert np.array_equal(got[:, 3] != 0, want[:, 3] != 0)
    assert np.abs(got[:, 3] - want[:, 3]).max() <= 1e-6 * np.abs(want[:, 3]).max()
    ai = np.loadtxt(os.path.join(str(tmp_path), "AiTable.dat"))
    assert np.allclose(ai, np.loadtxt(os.path.join(GOLDEN, "tables", name, "AiTable.dat")), rtol=1e-15, atol=1e-15)

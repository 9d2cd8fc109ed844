"""Golden values of the reference Decomposer's dense kernels, for the GPU
modal decomposition tests.

Builds the reference's Cython/C basis module in a scratch copy (the recipe of
make_alpha_tables.py) and stores, under tests/golden/decomp/:

  small_m6_k24.npz   a small Basis (mode_p_max 6, k_grid_size 24): the mode
                     bispectrum covariance from compute_mode_bispectra_covariance
                     (tetrapyd.c:107-236), QS from compute_QS (tetrapyd.c:
                     238-305) for two shapes, and np.linalg.cond of a few
                     bordered sub-blocks of the normalised covariance, as
                     get_cond computes them (cmbbest.pyx:44-47);
  scalarI_m10_L500_n256_S.npz
                     the ScalarI (mass 1) shape function on the k_grid_size 150
                     tetrapyd of the scalarI_m10_L500_n256 table, evaluated by
                     the reference's own model class, so that the GPU
                     decomposition of that table can be checked without the
                     reference at test time.

Usage: python tests/golden/make_decomp_fixtures.py   (needs the reference checkout)
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
OUT = os.path.join(HERE, "decomp")

from make_alpha_tables import build_reference  # noqa: E402


def main():
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        build_reference(tmp)
        os.environ.setdefault("TMPDIR", tmp)
        sys.path.insert(0, tmp)
        import Aarambam as Am  # noqa: E402  (the scratch copy)
        best = Am.basis.cmbbest

        kF = 2 * np.pi / 500.0
        b = best.Basis(mode_p_max=6, parameter_n_scalar=0.965, k_grid_size=24, k_min=kF, k_max=kF * 128)
        k1, k2, k3 = b.tetrapyd_grid
        ns = 0.965
        S = np.stack([k1 ** 2 * (k2 * k3) ** (ns - 2) + k2 ** 2 * (k3 * k1) ** (ns - 2) + k3 ** 2 * (k1 * k2) ** (ns - 2),
                      np.sin(3.0 * np.log(k1 + k2 + k3))])
        QS = b.compute_QS_C(S)
        QQ = b.mode_bispectra_covariance
        norms = np.sqrt(np.diag(QQ))
        QQt = QQ / norms[:, None] / norms[None, :]
        rng = np.random.default_rng(5)
        nm = QQ.shape[0]
        sets, conds = [], []
        for size in (4, 10, 20):
            msk = np.zeros(nm, dtype=bool)
            msk[rng.choice(nm, size, replace=False)] = True
            cand = np.where(~msk)[0]
            conds.append([best.get_cond(i, msk, QQt) for i in cand])
            sets.append(msk)
        np.savez_compressed(os.path.join(OUT, "small_m6_k24.npz"), QQ=QQ, QS=QS, S=S, masks=np.array(sets),
                            conds=np.concatenate([np.asarray(c, dtype=np.float64) for c in conds]),
                            k_grid=b.k_grid, k_weights=b.k_weights,
                            tetrapyd_indices=b.tetrapyd_indices, tetrapyd_grid_weights=b.tetrapyd_grid_weights,
                            mode_evals=b.mode_function_evaluations, mode_indices=b.mode_indices)
        print("small_m6_k24", QQ.shape, QS.shape)

        # ScalarI shape on the scalarI_m10_L500_n256 tetrapyd
        kF = 2 * np.pi / 500.0
        b = best.Basis(mode_p_max=10, parameter_n_scalar=0.965, k_grid_size=150, k_min=kF, k_max=kF * 256)
        C = type("C", (Am.models.ScalarI, Am.basis.BasicBasisDecompose), {})
        inst = C(N_modes=10, n_s=0.965, Lbox=500.0, Nmax=256, ModeTol=1e-4, MaxModeCount=150, mass=1.0)
        k1, k2, k3 = b.tetrapyd_grid
        S = inst.shape_function(k1, k2, k3)
        np.savez_compressed(os.path.join(OUT, "scalarI_m10_L500_n256_S.npz"), S=S,
                            tetrapyd_indices=b.tetrapyd_indices.astype(np.int16))
        print("scalarI_m10_L500_n256_S", S.shape)


if __name__ == "__main__":
    main()

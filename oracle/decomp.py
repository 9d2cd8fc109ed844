"""CPU oracle of the modal decomposition's dense kernels (test
infrastructure only; never imported by the package).

A plain numpy restatement, for small grids, of what the reference computes in
Aarambam/basis/tetrapyd.c and cmbbest.pyx:
  covariance(...)  QQ[n][m] = sum_t w_t Q_n(t) Q_m(t)   (tetrapyd.c:107-236)
  project(...)     QS[s][n] = sum_t S[s][t] w_t Q_n(t)  (tetrapyd.c:238-305)
  residual(...)    S - sum_j c_j Q_{sel_j}              (cmbbest.pyx:433)
  cond(...)        np.linalg.cond of a sub-block, as get_cond (cmbbest.pyx:44-47)
with Q_n(t) the symmetrised product of tetrapyd.c:136-152.  Pinned against
the reference's own compiled kernels through tests/golden/decomp/small_m6_k24.npz.
"""
import itertools

import numpy as np


def mode_bispectra(tetra_idx, mode_idx, mode_evals):
    """Q [n_modes][npts] (tetrapyd.c:136-152)."""
    i = tetra_idx
    p = mode_idx
    Q = np.zeros((p.shape[1], i.shape[1]))
    for a, b, c in itertools.permutations(range(3)):
        Q += mode_evals[p[0]][:, i[a]] * mode_evals[p[1]][:, i[b]] * mode_evals[p[2]][:, i[c]]
    return Q / 6.0


def covariance(w, tetra_idx, mode_idx, mode_evals):
    Q = mode_bispectra(tetra_idx, mode_idx, mode_evals)
    return (Q * w[None, :]) @ Q.T


def project(S, w, tetra_idx, mode_idx, mode_evals):
    Q = mode_bispectra(tetra_idx, mode_idx, mode_evals)
    return (np.atleast_2d(S) * w[None, :]) @ Q.T


def residual(S, sel, coef, tetra_idx, mode_idx, mode_evals):
    Q = mode_bispectra(tetra_idx, mode_idx, mode_evals)
    return S - np.sum(Q[sel] * np.asarray(coef)[:, None], axis=0)


def cond(i, msk, QQ_tilde):
    m = msk.copy()
    m[i] = True
    return np.linalg.cond(QQ_tilde[np.ix_(m, m)])

"""Loaders for the coefficient and transfer-function tables.

AlphaTable: lines "p q r alpha" (Aarambam/basis/decompose.py:318), read with
fscanf " %d %d %d %lf " and stored at all six index permutations
(Aarambam/LPT/Basis/main.c:213-247); entries may appear in any order, later
lines overwrite earlier ones.  AiTable (X0): lines "p x0 x1", column x0 used
(main.c:249-289).  Transfer table: two columns "k T" (power.c:66-153).
"""
from __future__ import annotations

import numpy as np


class TableError(Exception):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def _scan_rows(path: str, ncols: int, kinds: str):
    """fscanf-style scan: stop at the first row that does not convert."""
    try:
        with open(path, "r") as f:
            toks = f.read().split()
    except OSError:
        raise TableError(17, f"can't read coefficients in file '{path}'") from None
    rows = []
    for i in range(0, len(toks) - ncols + 1, ncols):
        chunk = toks[i:i + ncols]
        try:
            rows.append(tuple(int(c) if k == "i" else float(c) for c, k in zip(chunk, kinds)))
        except ValueError:
            break
    return rows


def load_alpha(path: str, n_modes: int) -> np.ndarray:
    """Symmetric alpha[M][M][M] float64 (main.c:215-241)."""
    a = np.zeros((n_modes, n_modes, n_modes), dtype=np.float64)
    for p, q, r, v in _scan_rows(path, 4, "iiif"):
        for (x, y, z) in ((r, q, p), (r, p, q), (q, r, p), (q, p, r), (p, r, q), (p, q, r)):
            if not (0 <= x < n_modes and 0 <= y < n_modes and 0 <= z < n_modes):
                raise TableError(17, f"alpha index ({p},{q},{r}) outside N_modes={n_modes}")
            a[x, y, z] = v
    if not np.all(np.isfinite(a)):
        raise TableError(17, "non-finite alpha coefficient")
    return a


def load_x0(path: str, n_modes: int) -> np.ndarray:
    """X0[M] (first value column of AiTable, main.c:250-289)."""
    x0 = np.zeros(n_modes, dtype=np.float64)
    for n, v0, _v1 in _scan_rows(path, 3, "iff"):
        if not (0 <= n < n_modes):
            raise TableError(17, f"X0 index {n} outside N_modes={n_modes}")
        x0[n] = v0
    return x0


def load_transfer(path: str):
    """(k, T) float64 columns of the tabulated transfer function."""
    rows = _scan_rows(path, 2, "ff")
    if not rows:
        raise TableError(17, f"can't read input transfer function in file '{path}'")
    arr = np.asarray(rows, dtype=np.float64)
    return arr[:, 0].copy(), arr[:, 1].copy()


def bbks_transfer(gamma: float = 0.21, kmin: float = 1e-5, kmax: float = 1e2, n: int = 2000):
    """BBKS transfer function T(q), q = k/Gamma, on log-spaced k (h/Mpc)."""
    k = np.logspace(np.log10(kmin), np.log10(kmax), n)
    q = k / gamma
    t = np.log(1 + 2.34 * q) / (2.34 * q) * (1 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3
                                          + (6.71 * q) ** 4) ** -0.25
    return k, t


def write_transfer(path: str, k, t) -> None:
    np.savetxt(path, np.column_stack([k, t]), fmt="%.17g")


def active_pairs(alpha: np.ndarray):
    """Sorted (p, q) pairs p <= q with some alpha[p][q][r] != 0, r >= q
    (the pairs the reference transforms, main.c:745-759)."""
    m = alpha.shape[0]
    return [(p, q) for p in range(m) for q in range(p, m) if np.any(alpha[p, q, q:] != 0)]

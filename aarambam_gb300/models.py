"""Bispectrum templates as model mix-ins for `utils.Decomposer`.

A model is a class defining `bispectrum(k1, k2, k3)` (the full, symmetric
bispectrum) or `raw_bispectrum(k1, k2, k3)` (one term, which
`basis.BasicBasisDecompose.bispectrum` sums over the six permutations), with
its parameters read from `self.args` (n_s and the model's own keywords given
to `Decomposer.go`).  That is the reference's plugin contract
(Aarambam/utils.py:409-446, Aarambam/models/*.py), so the reference's own
model classes plug into this package's Decomposer unchanged.

The templates here are the standard published forms in the reference's
conventions (a near-scale-invariant tilt through n_s; raw forms of rescaled
wavenumbers k^((4 - n_s)/3)):
  Local         Komatsu & Spergel 2001 (Aarambam/models/SingleField.py:5-27)
  Equilateral   Creminelli et al. 2006 (SingleField.py:30-78)
  Orthogonal    Senatore, Smith & Zaldarriaga 2010 (SingleField.py:81-130)
  LogResonance  log-oscillation template, Planck 2018 IX eq. 12
                (Aarambam/models/Resonances.py:3-31)
"""
from __future__ import annotations

import numpy as np


def _tilted(args, k1, k2, k3):
    """k_i^2, k_i^((n_s+2)/3), k_i^(2(n_s-1)/3), k_i^(n_s-2) for the three sides."""
    ns = args["n_s"]
    out = []
    for k in (k1, k2, k3):
        out.append((k * k, np.power(k, (ns + 2) / 3), np.power(k, 2 * (ns - 1) / 3), np.power(k, ns - 2)))
    return out


def _eq_orth(args, k1, k2, k3, c1, c2, c3):
    """c1 S_1 + c2 S_2 + c3 S_3 with S_1 the squeezed-type, S_2 the
    equilateral-type and S_3 the mixed sum of the equilateral/orthogonal
    templates, over (k1 k2 k3)^2."""
    (q1, l1, o1, n1), (q2, l2, o2, n2), (q3, l3, o3, n3) = _tilted(args, k1, k2, k3)
    s1 = q1 * n2 * n3 + q2 * n3 * n1 + q3 * n1 * n2
    s2 = o1 * o2 * o3
    s3 = n1 * o2 * l3 + n1 * o3 * l2 + n2 * o1 * l3 + n2 * o3 * l1 + n3 * o1 * l2 + n3 * o2 * l1
    return (c1 * s1 + c2 * s2 + c3 * s3) / (k1 * k2 * k3) ** 2


class Local:
    """Local-type template, normalised to 1 in the equilateral limit."""

    def bispectrum(self, k1, k2, k3):
        t = self.args["n_s"] - 2
        s = (k1 ** 2 * (k2 * k3) ** t + k2 ** 2 * (k3 * k1) ** t + k3 ** 2 * (k1 * k2) ** t) / 3
        return s / (k1 * k2 * k3) ** 2


class Equilateral:
    """Equilateral template (-1, -2, +1 combination)."""

    def bispectrum(self, k1, k2, k3):
        return _eq_orth(self.args, k1, k2, k3, -1, -2, 1)


class Orthogonal:
    """Orthogonal template (-3, -8, +3 combination)."""

    def bispectrum(self, k1, k2, k3):
        return _eq_orth(self.args, k1, k2, k3, -3, -8, 3)


class LogResonance:
    """sin(w_res ln(k1 + k2 + k3) + phi) in rescaled wavenumbers."""

    def raw_bispectrum(self, k1, k2, k3):
        e = (4 - self.args["n_s"]) / 3
        k1, k2, k3 = np.power(k1, e), np.power(k2, e), np.power(k3, e)
        s = np.sin(self.args["w_res"] * np.log(k1 + k2 + k3) + self.args["phi"]) * 1 / 6
        return s / (k1 * k2 * k3) ** 2

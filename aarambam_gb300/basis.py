"""Modal decomposition of a bispectrum template into the separable basis the
2LPT step reads (AlphaTable.dat / AiTable.dat), with the dense work on the GPU.

Interface of the reference's Aarambam.basis (cmbbest.pyx `Basis`, `Model`;
decompose.py `BasicBasisDecompose`): the same constructor arguments,
attributes, methods and outputs, so that `utils.Decomposer.go(Model,
BasicBasisDecompose)` runs unchanged with any model mix-in that defines
`bispectrum` or `raw_bispectrum` (this package's `models`, or the reference's
own Aarambam.models classes, which are plain numpy).

What runs where:
  host (numpy)  the 1D k grid and weights, the tetrapyd points, the 1D mode
                functions, the model's shape function, the conjugate-gradient
                solves (scipy, FP64) and the bookkeeping of the orthogonal
                matching pursuit;
  GPU           the mode bispectra Q_n(t) (FP64, made once per basis and
                kept on the device), the mode-bispectrum covariance QQ
                (tetrapyd.c:107-236) on the tensor cores, FP64-accurate (bf16
                digits, exact level sums), and in FP64 the projections QS / QR
                (tetrapyd.c:238-305, cmbbest.pyx:419-426, :459), the residual
                R on the tetrapyd (cmbbest.pyx:433) and
                one condition number per candidate mode and iteration
                (cmbbest.pyx:44-47, :443-446) from the bordered-matrix secular
                equation instead of an SVD per candidate
                (aarambam_gb300/csrc/decomp.cu).
The matching-pursuit loop itself follows cmbbest.pyx:320-490 step for step;
the diagnostic `prho` (cmbbest.pyx:441) is not computed (nothing reads it).
"""
from __future__ import annotations

import ctypes as C
import itertools
import time

import numpy as np
import torch
from scipy import special
from scipy.sparse.linalg import cg as conjugate_gradient

from . import _lib


def _ptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


class Basis:
    """The separable Legendre basis on a tetrapyd grid (cmbbest.pyx:50-101)."""

    def __init__(self, k_min, k_max, parameter_n_scalar, mode_p_max, k_grid_size, device=None, verbose=True,
                 host_only=False):
        self.mode_p_max = int(mode_p_max)
        self.parameter_n_scalar = parameter_n_scalar
        self.mode_k_min = k_min
        self.mode_k_max = k_max
        self.verbose = verbose
        self.mode_functions = self.legendre_basis()
        self.k_grid_size = int(k_grid_size)
        self.k_grid, self.k_weights = self.create_k_grid(grid_type="uniform")
        self.tetrapyd_indices, self.tetrapyd_grid = self.create_tetrapyd_grid()
        self.tetrapyd_grid_size = self.tetrapyd_grid.shape[1]
        w = np.prod(self.k_weights[self.tetrapyd_indices], axis=0)
        self.tetrapyd_grid_weights = w / np.sum(w)
        self.mode_function_evaluations = self.mode_functions(self.k_grid)
        self.mode_indices, self.mode_symmetry_factor = self.create_mode_indices()
        self.mode_bispectra_evaluations = None
        if host_only:  # grids and mode functions only (no covariance)
            return
        self.device = torch.device(device if device is not None else "cuda")
        self._upload()
        t0 = time.time()
        self.mode_bispectra_covariance = self.compute_mode_bispectra_covariance()
        self.mode_bispectra_norms = np.sqrt(np.diag(self.mode_bispectra_covariance))
        self.timings = {"covariance_s": time.time() - t0}
        if verbose:
            print(f"Basis is now ready ({self.mode_indices.shape[1]} modes, {self.tetrapyd_grid_size} tetrapyd "
                  f"points, covariance in {self.timings['covariance_s']:.2f} s on the GPU)")

    # ------------------------------------------------------------ host parts
    def legendre_basis(self):
        """Mode functions f_p(k) (cmbbest.pyx:103-142): monomials
        k^(2 + s (p - 3)) for p <= 3, shifted Legendre polynomials
        P_{p-1}(kbar) - P_{p-1}(kbar(0)) above, s = (4 - n_s) / 3."""
        n_s, kmin, kmax, pmax = self.parameter_n_scalar, self.mode_k_min, self.mode_k_max, self.mode_p_max
        s = (4 - n_s) / 3
        span = np.power(kmax, s) - np.power(kmin, s)

        def basis_function(k):
            k = np.asarray(k, dtype=np.float64)
            kbar = -1 + 2 / span * (np.power(k, s) - np.power(kmin, s))
            out = np.zeros((pmax, len(k)))
            for p in range(pmax):
                if p <= 3:
                    out[p] = np.power(k, 2 + s * (p - 3))
                else:
                    zero_point = -1 - 2 * np.power(kmin, s) / span
                    # the power-basis polynomial scipy builds, as the reference evaluates it
                    out[p] = special.legendre(p - 1)(kbar) - special.eval_legendre(p - 1, zero_point)
            return out

        return basis_function

    def create_k_grid(self, grid_type="uniform"):
        """Uniform 1D grid and its weights (cmbbest.pyx:146-166): 1/k below
        2 k_median and 1/sqrt(k) above it and below 2 k_min."""
        if grid_type != "uniform":
            raise ValueError(f"Grid type {grid_type} is currently unsupported")
        k = np.linspace(self.mode_k_min, self.mode_k_max, self.k_grid_size)
        kmed = np.sqrt(self.mode_k_min * self.mode_k_max)
        w = np.where(k > kmed * 2, 1 / np.sqrt(k), 1 / k)
        w[k < 2 * self.mode_k_min] = 1 / np.sqrt(k[k < 2 * self.mode_k_min])
        return k, w

    def create_tetrapyd_grid(self, include_borderline=False):
        """Points i1 >= i2 >= i3 of the 1D grid with k2 + k3 >= k1, in the
        order of the reference's nested loops (cmbbest.pyx:169-214)."""
        if include_borderline:
            raise ValueError("include_borderline is not supported")
        n = self.k_grid_size
        i1, i2, i3 = [], [], []
        for a in range(n):
            b, c = np.tril_indices(a + 1)  # b >= c, row-major: b slow, c fast
            i1.append(np.full(b.shape, a))
            i2.append(b)
            i3.append(c)
        i1, i2, i3 = np.concatenate(i1), np.concatenate(i2), np.concatenate(i3)
        k = self.k_grid
        keep = k[i2] + k[i3] >= k[i1]
        idx = np.stack([i1[keep], i2[keep], i3[keep]], axis=0)
        return idx, np.stack([k[idx[0]], k[idx[1]], k[idx[2]]], axis=0)

    def create_mode_indices(self, p_max=None):
        """3D mode indices p1 >= p2 >= p3 in C order and their symmetry
        factors (cmbbest.pyx:216-235)."""
        p_max = self.mode_p_max if p_max is None else p_max
        p = np.arange(p_max, dtype=np.dtype("i"))
        p1, p2, p3 = np.meshgrid(p, p, p, indexing="ij")
        keep = (p1 >= p2) & (p2 >= p3)
        p1, p2, p3 = p1[keep], p2[keep], p3[keep]
        sym = np.ones(p1.shape[0])
        sym[(p1 != p2) & (p2 != p3)] = 6
        sym[(p1 == p2) & (p2 != p3)] = 3
        sym[(p1 != p2) & (p2 == p3)] = 3
        return np.stack([p1, p2, p3], axis=0), sym

    def evaluate_modal_basis_on_grid(self, k1, k2, k3):
        """Symmetrised 3D mode functions on given (k1, k2, k3) (cmbbest.pyx:260-273)."""
        p1, p2, p3 = self.mode_indices
        e1, e2, e3 = self.mode_functions(k1), self.mode_functions(k2), self.mode_functions(k3)
        out = np.zeros((len(p1), *np.shape(k1)))
        for q1, q2, q3 in itertools.permutations([p1, p2, p3]):
            out = out + (e1[q1, :] * e2[q2, :] * e3[q3, :] / 6)
        return out

    def evaluate_modal_bispectra_on_grid(self, coeffs, k1, k2, k3):
        return np.matmul(coeffs, self.evaluate_modal_basis_on_grid(k1, k2, k3))

    # ------------------------------------------------------------ GPU parts
    def _upload(self):
        dev = self.device
        i1, i2, i3 = self.tetrapyd_indices
        p1, p2, p3 = self.mode_indices
        as_i = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(dev)
        as_d = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        self._d = dict(w=as_d(self.tetrapyd_grid_weights), i1=as_i(i1), i2=as_i(i2), i3=as_i(i3), p1=as_i(p1),
                       p2=as_i(p2), p3=as_i(p3), f=as_d(self.mode_function_evaluations))
        # the mode bispectra Q[n][t], made once and read by the covariance and
        # by every projection and residual of the matching pursuit
        d = self._d
        self._ldq = int(_lib.load().aar_tetra_modes_ld(self.tetrapyd_grid_size))
        self._Q = torch.empty((self.mode_indices.shape[1], self._ldq), dtype=torch.float64, device=dev)
        self._call("aar_tetra_modes", _ptr(self._Q), self._ldq, _ptr(d["i1"]), _ptr(d["i2"]), _ptr(d["i3"]),
                   self.tetrapyd_grid_size, _ptr(d["p1"]), _ptr(d["p2"]), _ptr(d["p3"]), self.mode_indices.shape[1],
                   _ptr(d["f"]), self.mode_p_max, self.k_grid_size, self._stream())

    def _tetra_args(self):
        d = self._d
        return (_ptr(d["w"]), _ptr(d["i1"]), _ptr(d["i2"]), _ptr(d["i3"]), self.tetrapyd_grid_size, _ptr(d["p1"]),
                _ptr(d["p2"]), _ptr(d["p3"]), self.mode_indices.shape[1], _ptr(d["f"]), self.mode_p_max,
                self.k_grid_size)

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _call(self, name, *args):
        L = _lib.load()
        with torch.cuda.device(self.device):
            rc = getattr(L, name)(*args)
        if rc != _lib.AAR_OK:
            raise _lib.AarError(rc, f"{name} failed")

    def compute_mode_bispectra_covariance(self):
        """QQ[n][m] = sum_t w_t Q_n(t) Q_m(t) (tetrapyd.c:107-236) on the GPU's
        tensor cores, FP64-accurate, from the stored mode bispectra."""
        L = _lib.load()
        nm = self.mode_indices.shape[1]
        nbytes = L.aar_modes_covariance_scratch_bytes(self.tetrapyd_grid_size, nm)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        qq = torch.empty((nm, nm), dtype=torch.float64, device=self.device)
        self._call("aar_modes_covariance", _ptr(qq), _ptr(self._Q), self._ldq, _ptr(self._d["w"]),
                   self.tetrapyd_grid_size, nm, _ptr(scratch), C.c_size_t(nbytes), self._stream())
        self._qq_dev = qq
        return qq.cpu().numpy()

    def _project_dev(self, X: torch.Tensor) -> torch.Tensor:
        X = X.to(self.device, torch.float64).contiguous()
        out = torch.empty((X.shape[0], self.mode_indices.shape[1]), dtype=torch.float64, device=self.device)
        self._call("aar_modes_project", _ptr(out), _ptr(X), X.shape[0], _ptr(self._d["w"]), _ptr(self._Q), self._ldq,
                   self.tetrapyd_grid_size, self.mode_indices.shape[1], self._stream())
        return out

    def compute_QS_C(self, S):
        """QS[s][n] = sum_t S_s(t) w_t Q_n(t) (tetrapyd.c:238-305), FP64 on the GPU."""
        S = np.atleast_2d(np.asarray(S, dtype=np.float64))
        return self._project_dev(torch.from_numpy(S)).cpu().numpy()

    def _residual_dev(self, S_dev, sel, coef):
        R = torch.empty_like(S_dev)
        n = len(sel)
        sel_d = torch.from_numpy(np.ascontiguousarray(sel, dtype=np.int32)).to(self.device) if n else None
        coef_d = torch.from_numpy(np.ascontiguousarray(coef, dtype=np.float64)).to(self.device) if n else None
        self._call("aar_modes_residual", _ptr(R), _ptr(S_dev), _ptr(sel_d) if n else None,
                   _ptr(coef_d) if n else None, n, _ptr(self._Q), self._ldq, self.tetrapyd_grid_size, self._stream())
        return R

    def _candidate_conds(self, qq_t_dev, msk):
        """cond of QQ~[m + {i}] for every i outside m (cmbbest.pyx:443-446),
        and cond of QQ~[m] itself."""
        sel = np.where(msk)[0]
        cand = np.where(~msk)[0]
        A = self._qq_tilde[np.ix_(sel, sel)]
        lam, V = np.linalg.eigh(A)
        a = np.abs(lam)
        cond_here = a.max() / a.min() if a.min() > 0 else np.inf
        sel_t = torch.from_numpy(sel).to(self.device)
        cand_t = torch.from_numpy(cand).to(self.device)
        B = qq_t_dev.index_select(0, sel_t).index_select(1, cand_t)
        Vd = torch.from_numpy(V).to(self.device)
        Z = (Vd.T @ B).T.contiguous()  # column i of V^T B as row i
        cvec = qq_t_dev.diagonal()[cand_t].contiguous()
        lam_d = torch.from_numpy(np.ascontiguousarray(lam)).to(self.device)
        out = torch.empty(len(cand), dtype=torch.float64, device=self.device)
        self._call("aar_bordered_cond", _ptr(out), _ptr(lam_d), len(sel), _ptr(Z), _ptr(cvec), len(cand),
                   self._stream())
        return cond_here, out.cpu().numpy()

    # ------------------------------------------------------------ expansion
    def basis_expansion(self, model_list, regularization=0, Niter=1e4, rtol=1e-12, bad_modes=False, RR_tol=1e-2,
                        cond_tol=1e9, max_modes=None):
        """Expand shape functions in the separable basis by orthogonal
        matching pursuit with conjugate-gradient solves (cmbbest.pyx:320-490).
        Returns (alpha, shape_covariance, convergence_correlation,
        convergence_MSE) as the reference does."""
        N_models = len(model_list)
        N_modes = self.mode_indices.shape[1]
        QQ = self.mode_bispectra_covariance
        norms = self.mode_bispectra_norms
        p1, p2, p3 = self.mode_indices
        w = self.tetrapyd_grid_weights
        k1, k2, k3 = self.tetrapyd_grid
        if max_modes is None:
            max_modes = p1.size
        S = np.stack([m.shape_function(k1, k2, k3) for m in model_list])
        shape_covariance = np.matmul(S * w[np.newaxis, :], S.T)
        QS = self.compute_QS_C(S)
        # modes taken out of the basis (cmbbest.pyx:404-426): their rows and
        # columns of QQ and their projections are zeroed, the diagonal kept
        badmask = (((p1 <= 2) & (p2 == 0) & (p3 == 0)) | ((p1 == 1) & (p2 == 1) & (p3 == 0)))
        badmask |= bad_modes
        badinds = np.where(badmask)[0]
        if self.verbose:
            print("Zeroing out mode inds", badinds, "\n")
        QQ_temp = QQ * 1
        QS_temp = QS * 1
        for bi in badinds:
            QQ_temp[bi, :] = 0
            QQ_temp[:, bi] = 0
            QQ_temp[bi, bi] = QQ[bi, bi]
            QS_temp[:, bi] = 0
        QQ_tilde = QQ_temp / norms[:, np.newaxis] / norms[np.newaxis, :]
        qq_t_dev = torch.from_numpy(QQ_tilde).to(self.device)
        self._qq_tilde = QQ_tilde
        good = ~badmask
        alpha = np.zeros((N_models, N_modes))
        S_dev = torch.from_numpy(np.ascontiguousarray(S[0:1])).to(self.device)
        w_dev = self._d["w"]
        self.omp_log = []
        for model_no in range(N_models):
            QS_tilde = QS_temp[model_no, :] / norms
            msk = np.zeros_like(p1, dtype=bool)
            msk[(p1 <= 3) & (p2 <= 3) & (p3 <= 3)] = True
            if max_modes == -1:
                msk = np.ones_like(msk, dtype=bool)
            it = 0
            t0 = time.time()
            tp = dict.fromkeys(("cg", "residual", "cond", "project"), 0.0)  # seconds per pursuit phase
            while True:
                if len(norms) <= np.sum(msk):
                    break
                ix = np.ix_(msk, msk)
                ta = time.perf_counter()
                alpha_tmp, _ = conjugate_gradient(QQ_tilde[ix] + np.eye(np.sum(msk)) * regularization, QS_tilde[msk],
                                                  rtol=rtol, atol=0, maxiter=int(Niter))
                tb = time.perf_counter()
                # residual of the first shape on the tetrapyd (the reference
                # subtracts from every row of S and reads element [0, 0])
                sel = np.where(msk)[0]
                use = good[sel]
                R = self._residual_dev(S_dev, sel[use], (alpha_tmp / norms[sel])[use])
                RR = float(torch.sum(R * R * w_dev))
                tc = time.perf_counter()
                tp["cg"] += tb - ta
                tp["residual"] += tc - tb
                delta_RR = RR / shape_covariance
                if np.abs(delta_RR[0, 0]) <= RR_tol:
                    if self.verbose:
                        print(f"\n HIT LIMIT OF VAR_RES/VAR_TOT = {RR_tol:0.4e}. ENDING SEARCH", flush=True)
                    break
                if np.sum(msk) == max_modes - 1:
                    if self.verbose:
                        print("\n USED ALL AVAILABLE MODES", flush=True)
                    break
                ta = time.perf_counter()
                cond_here, cond = self._candidate_conds(qq_t_dev, msk)
                tp["cond"] += time.perf_counter() - ta
                fcond = cond / cond_here - 1
                if cond_here > cond_tol:
                    if self.verbose:
                        print(f"\n HIT LIMIT OF COND NUM {cond_here:0.4e} > {cond_tol:0.4e}. ENDING SEARCH", flush=True)
                    break
                ta = time.perf_counter()
                QR = self._project_dev(R)[0].cpu().numpy() / norms / np.sqrt(RR)
                tp["project"] += time.perf_counter() - ta
                QR[badinds] = 0
                QR = QR[np.invert(msk)]
                m = np.argsort(np.abs(QR))[-10:]
                m = m[np.argmin(fcond[m])]
                m = np.where(np.invert(msk))[0][m]
                msk[m] = True
                it += 1
                self.omp_log.append((it, float(delta_RR[0, 0]), float(cond_here), int(m)))
            self.timings.update({f"pursuit_{k}_s": v for k, v in tp.items()})
            self.timings["pursuit_s"] = time.time() - t0
            if self.verbose:
                print(f"\n USING MODES {np.where(msk)[0]} ({it} pursuit steps in {time.time() - t0:.2f} s)")
            alpha_tmp, _ = conjugate_gradient(QQ_tilde[np.ix_(msk, msk)] + np.eye(np.sum(msk)) * regularization,
                                              QS_tilde[msk], rtol=1e-16, atol=0, maxiter=int(1e6))
            alpha_tilde = np.zeros_like(norms)
            alpha_tilde[msk] = alpha_tmp
            alpha[model_no, :] = alpha_tilde / norms
        sum_SS = np.diag(shape_covariance)
        sum_SR = np.sum(alpha * QS, axis=1)
        sum_RR = np.sum(alpha * np.matmul(alpha, QQ), axis=1)
        corr = sum_SR / np.sqrt(sum_SS * sum_RR)
        corr = 1.0 - np.abs(1 - corr)
        mse = np.abs(sum_SS + sum_RR - 2 * sum_SR) / sum_SS
        return alpha, shape_covariance, corr, mse


class Model:
    """A bispectrum shape for `Basis.basis_expansion` (cmbbest.pyx:537-591,
    the "custom" form): shape_function(k1, k2, k3) = (k1 k2 k3)^2 B(k1, k2, k3)."""

    def __init__(self, shape_type, **kwargs):
        self.shape_type = shape_type.lower()
        if self.shape_type != "custom":
            raise ValueError("only shape_type='custom' (a given shape_function) is supported")
        self.shape_name = kwargs.get("shape_name", "custom")
        self.shape_function = kwargs["shape_function"]


class BasicBasisDecompose:
    """Modal decomposition of a model's bispectrum (decompose.py:5-321), the
    dense work on the GPU (see the module docstring).  Combined with a model
    mix-in by `utils.Decomposer`; reads N_modes, n_s, Lbox, Nmax, ModeTol,
    MaxModeCount (and the model's parameters) from self.args."""

    k_grid_size = 150

    def __init__(self, N_modes, n_s, Lbox, Nmax, ModeTol, MaxModeCount, **kwargs):
        args = dict(N_modes=N_modes, n_s=n_s, Lbox=Lbox, Nmax=Nmax, ModeTol=ModeTol, MaxModeCount=MaxModeCount)
        args.update(**kwargs)
        self.args = args

    def go(self):
        out = {}
        out.update(self.generate_alpha(verbose=self.args.get("verbose", True)))
        out.update(self.generate_Ai())
        return out

    def make_basis(self):
        kF = 2 * np.pi / self.args["Lbox"]
        return Basis(mode_p_max=self.args["N_modes"], parameter_n_scalar=self.args["n_s"],
                     k_grid_size=self.k_grid_size, k_min=kF, k_max=kF * self.args["Nmax"],
                     device=self.args.get("device"), verbose=self.args.get("verbose", True))

    def generate_alpha(self, verbose=True):
        """Coefficients alpha of the expansion (decompose.py:84-173)."""
        basis = self.make_basis()
        p1, p2, p3 = basis.mode_indices
        # low orders: keep only the three needed ones (decompose.py:122-128)
        msk = ((p1 < 4) & np.invert(((p1 == 1) & (p2 == 1) & (p3 == 1)) | ((p1 == 2) & (p2 == 1) & (p3 == 0)) |
                                     ((p1 == 3) & (p2 == 0) & (p3 == 0))))
        model = [Model(shape_type="custom", shape_name="TMP", shape_function=self.shape_function)]
        alpha, shape_cov, converg, converg_MSE = basis.basis_expansion(
            model, rtol=1e-10, Niter=1e3, bad_modes=msk, RR_tol=self.args["ModeTol"],
            max_modes=self.args["MaxModeCount"])
        eps = np.sqrt(2 * (1 - converg[0] ** 2))
        if verbose:
            print("\n-------------- BASIS DECOMPOSITION --------------")
            print("correlation : %0.10f (std = %0.8e, eps = %0.8e)" % (converg[0], np.sqrt(converg_MSE[0]), eps))
            print("-------------------------------------------------\n")
        kF = 2 * np.pi / self.args["Lbox"]
        kbin = np.geomspace(kF, kF * self.args["Nmax"] / 2, 100)
        ones = kF * np.ones_like(kbin)
        triples = [(kbin, kbin, ones), (kbin, kbin, kbin), (kbin, kbin, 2 * kbin)]
        Orig = np.vstack([self.shape_function(*t) for t in triples]).T
        Aprx = np.vstack([basis.evaluate_modal_bispectra_on_grid(alpha, *t) for t in triples]).T
        Templates = np.array([basis.evaluate_modal_basis_on_grid(*t) for t in triples])
        Aprx_split = alpha[0][None, :, None] * Templates
        self.basis = basis
        return dict(S_original=Orig, S_apprx=Aprx, Templates=Templates, kbin=kbin,
                    AlphaTable=np.vstack([basis.mode_indices, alpha[0]]).T, S_apprx_individual=Aprx_split)

    def generate_Ai(self):
        """X0 table: P_p(kbar(0)) per mode (decompose.py:176-216)."""
        scale = (4 - self.args["n_s"]) / 3
        kmin = 2 * np.pi / self.args["Lbox"]
        kmax = kmin * self.args["Nmax"]
        a, b = np.power(kmin, scale), np.power(kmax, scale)
        x0 = np.zeros([self.args["N_modes"], 2])
        for p in range(self.args["N_modes"]):
            x0[p, 0] = special.eval_legendre(p, -1 - 2 * a / (b - a))
        return {"AiTable": np.vstack([range(self.args["N_modes"]), x0.T]).T}

    def shape_function(self, k1, k2, k3):
        """(k1 k2 k3)^2 B(k1, k2, k3) (decompose.py:219-237)."""
        return self.bispectrum(k1, k2, k3) * (k1 * k2 * k3) ** 2

    def bispectrum(self, k1, k2, k3):
        """raw_bispectrum summed over the permutations of (k1, k2, k3)
        (decompose.py:240-275); models may define bispectrum directly."""
        if not hasattr(self, "raw_bispectrum"):
            raise NotImplementedError("Bispectrum not implemented. Must define `raw_bispectrum` method.")
        k = np.stack([k1, k2, k3])
        B = 0
        for a, b, c in itertools.permutations(range(3)):
            B += self.raw_bispectrum(k[a], k[b], k[c])
        return B

    def finalize(self, out, directory):
        """AlphaTable.dat (p1 p2 p3 alpha) and AiTable.dat (p x0 x1)
        (decompose.py:297-321)."""
        np.savetxt(directory + "/AlphaTable.dat", out["AlphaTable"], fmt="%d %d %d %.17g")
        np.savetxt(directory + "/AiTable.dat", out["AiTable"], fmt="%d %.17g %.17g")
        print(f"Tables written out to {directory}")

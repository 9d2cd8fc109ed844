"""ctypes wrapper around the FP64 C oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.  `build()` compiles oracle/aar_oracle.c with the
Makefile beside it; nothing here is loaded by the product library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "2LPTBasis")

_lib = None


def build(ref: bool = False) -> None:
    subprocess.check_call(["make", "-s", "-C", HERE, "all"] + (["ref", "REF=" + reference_checkout()] if ref else []))


def reference_checkout() -> str:
    """Directory the Makefile's `ref` target compiles the reference from:
    $AARAMBAM_REFERENCE when set, else the Makefile's default."""
    env = os.environ.get("AARAMBAM_REFERENCE")
    if env:
        return env
    out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return out.stdout.strip()


def reference_present() -> bool:
    """True when the reference's 2LPT sources can be compiled here."""
    d = reference_checkout()
    return bool(d) and os.path.isfile(os.path.join(d, "Aarambam", "LPT", "Basis", "main.c"))


class Cosmo(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "Omega", "OmegaLambda", "HubbleParam", "Sigma8", "PrimordialIndex", "Redshift",
        "UnitLength_in_cm", "UnitMass_in_g", "UnitVelocity_in_cm_per_s", "InputSpectrum_UnitLength_in_cm")]


class Params(C.Structure):
    _fields_ = [("N", C.c_int), ("Nsample", C.c_int), ("Nmax", C.c_int), ("Seed", C.c_int),
                ("Box", C.c_double), ("ns", C.c_double), ("Fnl", C.c_double),
                ("FixedAmplitude", C.c_int), ("PhaseFlip", C.c_int), ("SphereMode", C.c_int)] + \
               [(n, C.c_double) for n in ("Norm", "Anorm", "D0", "Dplus", "InitTime", "Hubble", "Beta",
                                          "vel_prefac", "vel_prefac2", "kconv")] + \
               [("ntrans", C.c_int), ("logk", C.POINTER(C.c_double)), ("logT", C.POINTER(C.c_double))] + \
               [("ResBasis", C.c_int), ("WhichSpectrum", C.c_int)] + \
               [(n, C.c_double) for n in ("A_res", "w_res", "phi_res")]


class Rlx(C.Structure):
    _fields_ = [("x", C.c_int64 * 12), ("carry", C.c_int64), ("pos", C.c_int), ("luxury", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C")
        fp = np.ctypeslib.ndpointer(np.float32, flags="C")
        up = np.ctypeslib.ndpointer(np.uint32, flags="C")
        L.orc_rlx_seed.argtypes = [C.POINTER(Rlx), C.c_ulong, C.c_int]
        L.orc_rlx_uniform.argtypes = [C.POINTER(Rlx)]
        L.orc_rlx_uniform.restype = C.c_double
        L.orc_rlx_get.argtypes = [C.POINTER(Rlx)]
        L.orc_rlx_get.restype = C.c_ulong
        L.orc_setup.argtypes = [C.POINTER(Params), C.POINTER(Cosmo), C.c_int, dp, dp]
        L.orc_setup.restype = C.c_int
        L.orc_free.argtypes = [C.POINTER(Params)]
        L.orc_transfer.argtypes = [C.POINTER(Params), C.c_double]
        L.orc_transfer.restype = C.c_double
        L.orc_c2r_3d.argtypes = [C.c_int, dp, dp]
        L.orc_r2c_3d.argtypes = [C.c_int, dp, dp]
        L.orc_seedtable.argtypes = [C.c_int, C.c_int, up]
        L.orc_gauss_potential.argtypes = [C.POINTER(Params), up, dp]
        L.orc_modal_acc.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, dp]
        L.orc_modal_acc_regrouped.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp,
                                              np.ctypeslib.ndpointer(np.int32, flags="C"), dp]
        L.orc_combine.argtypes = [C.POINTER(Params), dp, dp, C.c_void_p, C.c_void_p]
        L.orc_lpt_fields.argtypes = [C.POINTER(Params), dp, dp]
        L.orc_readout.argtypes = [C.POINTER(Params), dp, C.c_int64, fp, fp]
        L.orc_tile_glass.argtypes = [C.POINTER(Params), fp, C.c_int64, C.c_double, C.c_int, fp, C.c_void_p]
        _lib = L
    return _lib


class Ranlux:
    """GSL ranlxd1/ranlxd2 restatement."""

    def __init__(self, seed: int, luxury: int = 202):
        self.s = Rlx()
        lib().orc_rlx_seed(C.byref(self.s), seed, luxury)

    def uniform(self) -> float:
        return lib().orc_rlx_uniform(C.byref(self.s))

    def get(self) -> int:
        return lib().orc_rlx_get(C.byref(self.s))


class Oracle:
    """The FP64 path for one configuration (dict of parameter-file values)."""

    def __init__(self, cfg: dict, k: np.ndarray, T: np.ndarray):
        c = Cosmo(Omega=cfg["Omega"], OmegaLambda=cfg["OmegaLambda"], HubbleParam=cfg["HubbleParam"],
                  Sigma8=cfg["Sigma8"], PrimordialIndex=cfg["PrimordialIndex"], Redshift=cfg["Redshift"],
                  UnitLength_in_cm=cfg["UnitLength_in_cm"], UnitMass_in_g=cfg["UnitMass_in_g"],
                  UnitVelocity_in_cm_per_s=cfg["UnitVelocity_in_cm_per_s"],
                  InputSpectrum_UnitLength_in_cm=cfg["InputSpectrum_UnitLength_in_cm"])
        p = Params(N=cfg["Nmesh"], Nsample=cfg["Nsample"], Nmax=cfg["Nmax"], Seed=cfg["Seed"], Box=cfg["Box"],
                   ns=cfg["PrimordialIndex"], Fnl=cfg["Fnl"], FixedAmplitude=cfg["FixedAmplitude"],
                   PhaseFlip=cfg["PhaseFlip"], SphereMode=cfg["SphereMode"])
        if "A_res" in cfg:  # a 2LPTResBasis parameter set
            p.ResBasis, p.WhichSpectrum = 1, cfg["WhichSpectrum"]
            p.A_res, p.w_res, p.phi_res = cfg["A_res"], cfg["w_res"], cfg["phi_res"]
        rc = lib().orc_setup(C.byref(p), C.byref(c), len(k), np.ascontiguousarray(k, np.float64),
                             np.ascontiguousarray(T, np.float64))
        if rc != 0:
            raise RuntimeError(f"oracle set-up failed with code {rc}")
        self.p = p
        self.N = cfg["Nmesh"]

    def __del__(self):
        try:
            lib().orc_free(C.byref(self.p))
        except Exception:
            pass

    @property
    def scalars(self) -> dict:
        return {n: getattr(self.p, n) for n in ("Norm", "Anorm", "D0", "Dplus", "InitTime", "Hubble", "Beta",
                                                "vel_prefac", "vel_prefac2")}

    def seedtable(self) -> np.ndarray:
        t = np.zeros(self.N * self.N, dtype=np.uint32)
        lib().orc_seedtable(self.p.Seed, self.N, t)
        return t.reshape(self.N, self.N)

    def gauss(self, seedtable=None) -> np.ndarray:
        N = self.N
        st = self.seedtable() if seedtable is None else seedtable
        out = np.zeros((N, N, N // 2 + 1, 2), dtype=np.float64)
        lib().orc_gauss_potential(C.byref(self.p), np.ascontiguousarray(st, np.uint32).ravel(), out.reshape(-1))
        return out

    def modal_acc(self, alpha: np.ndarray, x0: np.ndarray, phik: np.ndarray) -> np.ndarray:
        N = self.N
        out = np.zeros((N, N, N // 2 + 1, 2), dtype=np.float64)
        M = alpha.shape[0]
        lib().orc_modal_acc(C.byref(self.p), M, np.ascontiguousarray(alpha, np.float64).ravel(),
                            np.ascontiguousarray(x0, np.float64), np.ascontiguousarray(phik).reshape(-1),
                            out.reshape(-1))
        return out

    def modal_acc_regrouped(self, alpha: np.ndarray, x0: np.ndarray, phik: np.ndarray, r_on=None) -> np.ndarray:
        """The regrouped accumulation over the radial modes r with r_on[r]
        (all when None): one part's share of a modal sum split over r."""
        N = self.N
        M = alpha.shape[0]
        on = np.ones(M, np.int32) if r_on is None else np.ascontiguousarray(r_on, np.int32)
        out = np.zeros((N, N, N // 2 + 1, 2), dtype=np.float64)
        lib().orc_modal_acc_regrouped(C.byref(self.p), M, np.ascontiguousarray(alpha, np.float64).ravel(),
                                      np.ascontiguousarray(x0, np.float64), np.ascontiguousarray(phik).reshape(-1),
                                      on, out.reshape(-1))
        return out

    def combine(self, phik: np.ndarray, acc: np.ndarray, want_pot: bool = False):
        N = self.N
        ph = np.array(phik, dtype=np.float64, copy=True)
        pg = np.zeros((N, N, N)) if want_pot else None
        pn = np.zeros((N, N, N)) if want_pot else None
        lib().orc_combine(C.byref(self.p), ph.reshape(-1), np.ascontiguousarray(acc).reshape(-1),
                          pg.ctypes.data if want_pot else None, pn.ctypes.data if want_pot else None)
        return (ph, pg, pn) if want_pot else ph

    def lpt_fields(self, phik: np.ndarray) -> np.ndarray:
        N = self.N
        out = np.zeros((6, N, N, N), dtype=np.float64)
        lib().orc_lpt_fields(C.byref(self.p), np.ascontiguousarray(phik).reshape(-1), out.reshape(-1))
        return out

    def readout(self, disp: np.ndarray, pos: np.ndarray):
        pos = np.array(pos, dtype=np.float32, copy=True).reshape(-1)
        vel = np.zeros_like(pos)
        lib().orc_readout(C.byref(self.p), np.ascontiguousarray(disp).reshape(-1), pos.size // 3, pos, vel)
        return pos.reshape(-1, 3), vel.reshape(-1, 3)

    def tile_glass(self, glass: np.ndarray, glass_box: float, tile: int) -> np.ndarray:
        g = np.ascontiguousarray(glass, np.float32).reshape(-1)
        n = g.size // 3
        out = np.zeros(n * tile**3 * 3, dtype=np.float32)
        lib().orc_tile_glass(C.byref(self.p), g, n, glass_box, tile, out, None)
        return out.reshape(-1, 3)

    def run(self, alpha, x0, lagr_pos):
        """Whole path; returns dict of intermediates and particles."""
        st = self.seedtable()
        g = self.gauss(st)
        acc = self.modal_acc(alpha, x0, g)
        tot, pot_g, pot_ng = self.combine(g, acc, want_pot=True)
        disp = self.lpt_fields(tot)
        pos, vel = self.readout(disp, lagr_pos)
        return dict(seedtable=st, gauss=g, acc=acc, total=tot, pot_gauss=pot_g, pot_ng=pot_ng, disp=disp,
                    pos=pos, vel=vel)


def c2r(c: np.ndarray) -> np.ndarray:
    N = c.shape[0]
    out = np.zeros((N, N, N))
    lib().orc_c2r_3d(N, np.ascontiguousarray(c, np.float64).reshape(-1), out.reshape(-1))
    return out


def r2c(r: np.ndarray) -> np.ndarray:
    N = r.shape[0]
    out = np.zeros((N, N, N // 2 + 1, 2))
    lib().orc_r2c_3d(N, np.ascontiguousarray(r, np.float64).reshape(-1), out.reshape(-1))
    return out

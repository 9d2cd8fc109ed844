"""Shared helpers for the tests: golden cases, tables, oracle runs."""
import functools
import json
import os

import numpy as np

from aarambam_gb300 import gadget, tables

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = ["local_n32", "scalarI_n32_flip_fixed_cut", "scalarI12_n16_sphere", "local_n24"]
# 2LPTResBasis outputs (oscillating P(k)): WhichSpectrum 1, 2 and 0
RES_CASES = ["res_lin_n32", "res_log_n32", "res_both_n16"]

BASE_CFG = dict(Omega=0.3, OmegaLambda=0.7, OmegaBaryon=0.0, OmegaDM_2ndSpecies=0.0, HubbleParam=0.7,
                ShapeGamma=0.0, Sigma8=0.8, PrimordialIndex=0.965, Redshift=49.0, FixedAmplitude=0, PhaseFlip=0,
                SphereMode=0, SavePotentialField=0, WhichSpectrum=0, WhichTransfer=2,
                InputSpectrum_UnitLength_in_cm=3.085678e24, UnitLength_in_cm=3.085678e24,
                UnitMass_in_g=1.989e43, UnitVelocity_in_cm_per_s=1e5)


def load_case(name):
    z = np.load(os.path.join(GOLDEN, "ref", name + ".npz"))
    cfg = json.loads(str(z["config"]))
    return cfg, z


@functools.lru_cache(maxsize=None)
def table(name, M):
    d = os.path.join(GOLDEN, "tables", name)
    return tables.load_alpha(os.path.join(d, "AlphaTable.dat"), M), tables.load_x0(os.path.join(d, "AiTable.dat"), M)


@functools.lru_cache(maxsize=None)
def bbks():
    return tables.bbks_transfer()


def make_cfg(N, Box, Seed, Fnl, M, table_name, Nmax, Nsample=None, **kw):
    cfg = dict(BASE_CFG)
    cfg.update(Nmesh=N, Nsample=Nsample or N, Nmax=Nmax, Box=Box, Seed=Seed, Fnl=Fnl, N_modes=M, table=table_name)
    cfg.update(kw)
    return cfg


def lattice_lagrangian(oracle, n_glass, tile):
    glass = gadget.lattice_glass(n_glass, 100.0)
    return oracle.tile_glass(glass, 100.0, tile)


def rel_rms(a, b):
    a, b = np.asarray(a), np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a, b = a.astype(dt), b.astype(dt)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def periodic_delta(p, q, box):
    d = np.asarray(p, np.float64) - np.asarray(q, np.float64)
    return d - box * np.round(d / box)

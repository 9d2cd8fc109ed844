"""Configuration and post-processing helpers with the reference's interface
(Aarambam/utils.py): make_config_basis / make_config_resbasis and their
make_example_config_* build the 2LPT parameter file text, collate_potential
gathers the potential dumps, camb2input converts a CAMB transfer file, and
Decomposer runs the modal decomposition that writes the coefficient tables.

Differences, deliberately: the default OutputDir comes from TMPDIR when set
and the system temporary directory otherwise (the reference raises KeyError
at import without TMPDIR, utils.py:61), and collate_potential also accepts the
single-file dumps a one-process run writes (`Gauss_potential_<Seed>`, whose
name the reference's collate mistakes for a slab size, utils.py:327), and
DEFAULT_RESBASIS_INPUTS carries Pk_mode = 1 (the reference's lacks the key,
so its make_example_config_resbasis raises TypeError).
"""
from __future__ import annotations

import gc
import glob
import os
import tempfile

import numpy as np

from . import gadget

DEFAULT_BASIS_CONFIG = """
Nmesh                               %(Nmesh)d
Nsample                             %(Nsample)d
Nmax                                %(Nmax)d
Box                                 %(Lbox)f
FileBase                            %(FileBase)s
OutputDir                           %(OutputDir)s
GlassFile                           %(GlassFile)s 
GlassTileFac                        %(GlassTileFac)d

Seed                                %(seed)d


Omega                               %(Om)f
OmegaLambda                         %(Ode)f
OmegaBaryon                         0.00000 #Doesn't really matter since we use the transfer function from CAMB
OmegaDM_2ndSpecies                  0.00
HubbleParam                         %(h)f
Sigma8                              %(sigma8)f
PrimordialIndex                     %(n_s)f
Redshift                            %(z_ini)f
Fnl                                 %(Fnl)f
N_modes                             %(N_modes)d


FixedAmplitude                      0
PhaseFlip                           0
SphereMode                          0
SavePotentialField                  %(SavePotentialField)d

WhichSpectrum                       0 #Fixed to 0 because we always want to use only the Transfer Function
WhichTransfer                       2 #Fixed to 2 because we always want a tabulated Transfer function (from CAMB)

FileWithInputSpectrum               ThisIsAFakeStringThatIsNeverUsed
FileWithInputTransfer               %(TransferPath)s
FileWithAlphaCoeff                  %(AlphaPath)s
FileWithX0Coeff                     %(AiPath)s

NumFilesWrittenInParallel           %(NWriteoutProcesses)d

InputSpectrum_UnitLength_in_cm      3.085678e24 #One Mpc in cm. This is fixed
UnitLength_in_cm                    3.085678e24 #One Mpc in cm, units of  Pkdgrav (gadget uses kpc)
UnitMass_in_g                       1.989e43
UnitVelocity_in_cm_per_s            1e5

ShapeGamma                          0.0    #Dont use this but it complains if I dont include it.
WDM_On                              0
WDM_Vtherm_On                       0
WDM_PartMass_in_kev                 10.0
"""

DEFAULT_BASIS_INPUTS = dict(Nmesh=256, Nsample=256, Nmax=256, Lbox=512, FileBase="Aarambam_ics",
                            OutputDir=os.environ.get("TMPDIR", tempfile.gettempdir()),
                            GlassFile="dummy_glass_dmonly_64.dat", GlassTileFac=4, seed=42, Om=0.3, Ode=0.7,
                            h=0.7, sigma8=0.8, n_s=0.96, z_ini=49, Fnl=100, N_modes=15,
                            TransferPath="TransferFunctionConverted.dat", AlphaPath="AlphaTable.dat",
                            AiPath="AiTable.dat", SavePotentialField=True, NWriteoutProcesses=os.cpu_count())


def make_config_basis(Nmesh, Nsample, Nmax, Lbox, FileBase, OutputDir, GlassFile, GlassTileFac, seed, Om, Ode, h,
                      sigma8, n_s, z_ini, Fnl, N_modes, TransferPath, AlphaPath, AiPath, SavePotentialField,
                      NWriteoutProcesses):
    """The 2LPT parameter-file text for these settings (utils.py:86-169)."""
    SavePotentialField = int(SavePotentialField)
    return DEFAULT_BASIS_CONFIG % locals()


def make_example_config_basis():
    return make_config_basis(**DEFAULT_BASIS_INPUTS)


# 2LPTResBasis: the Basis file with WhichSpectrum = Pk_mode and the three
# oscillation tags (utils.py:71-84)
DEFAULT_RESBASIS_CONFIG = (DEFAULT_BASIS_CONFIG + """
A_res               %(Pk_A_res)f
w_res               %(Pk_w_res)f
phi_res             %(Pk_phi_res)f
""").replace("0 #Fixed to 0 because we always want to use only the Transfer Function", "%(Pk_mode)d")

DEFAULT_RESBASIS_INPUTS = dict(DEFAULT_BASIS_INPUTS, Pk_A_res=0.9, Pk_w_res=2, Pk_phi_res=0.0, Pk_mode=1)


def make_config_resbasis(Nmesh, Nsample, Nmax, Lbox, FileBase, OutputDir, GlassFile, GlassTileFac, seed, Om, Ode,
                         h, sigma8, n_s, z_ini, Fnl, N_modes, TransferPath, AlphaPath, AiPath, SavePotentialField,
                         NWriteoutProcesses, Pk_A_res, Pk_w_res, Pk_phi_res, Pk_mode):
    """The 2LPTResBasis parameter-file text (utils.py:172-271).  Pk_mode is
    WhichSpectrum: the executable applies (1 + A cos(w k + phi)) and
    (1 + A cos(w ln k + phi)) for modes 0 and 1 and the log one only for 2
    (its switch has no break, ResBasis/main.c:445-455)."""
    SavePotentialField = int(SavePotentialField)
    return DEFAULT_RESBASIS_CONFIG % locals()


def make_example_config_resbasis():
    return make_config_resbasis(**DEFAULT_RESBASIS_INPUTS)


def camb2input(path):
    """(k, T) columns of a CAMB transfer file (utils.py:287-304)."""
    return np.loadtxt(path, usecols=[0, 6])


def collate_potential(OutputDir):
    """Gather the Gauss/Nongauss potential dumps of a run into [N, N, N]
    arrays (utils.py:307-346); the dump files are removed, as in the
    reference.  Accepts multi-slab names (..._StartX_<x>_NumX_<n>) and the
    single-file name a one-process run writes."""
    out = {}
    for t in ["Gauss_potential", "Nongauss_potential"]:
        files = sorted(f for f in glob.glob(os.path.join(OutputDir, f"{t}_*")) if not f.endswith(".npy"))
        if not files:
            continue
        slabs = []
        for fn in files:
            field, n, box = gadget.read_potential(fn) if "_StartX_" not in fn else (None, None, None)
            if field is None:
                rec = np.memmap(fn, offset=16, dtype=gadget.POT_DTYPE, mode="r")
                with open(fn, "rb") as f:
                    n = int(np.frombuffer(f.read(8), dtype="<i4")[1])
                nx = int(fn.split("_")[-1])
                field = np.array(rec["val"]).reshape(nx, n, n)
                del rec
            slabs.append(field)
            gc.collect()
            os.remove(fn)
        out[t] = np.concatenate(slabs, axis=0)
    return out


class Decomposer:
    """Bispectrum modal decomposition driver (utils.py:349-446): combines a
    model mix-in (models.py, or any class with `bispectrum` /
    `raw_bispectrum` reading self.args, e.g. the reference's own
    Aarambam.models classes) with a basis class (default
    basis.BasicBasisDecompose, whose dense FP64 work runs on the GPU), runs
    it and, with `outdir`, writes AlphaTable.dat / AiTable.dat there."""

    def __init__(self, N_modes, n_s, Lbox, Nmax, ModeTol, MaxModeCount, **kwargs):
        args = dict(N_modes=N_modes, n_s=n_s, Lbox=Lbox, Nmax=Nmax, ModeTol=ModeTol, MaxModeCount=MaxModeCount)
        args.update(**kwargs)
        self.args = args

    def go(self, Model, Basis=None, outdir=None, **kwargs):
        if Basis is None:
            from .basis import BasicBasisDecompose as Basis
        inpars = self.args.copy()
        inpars.update(**kwargs)
        decomp = type("C", (Model, Basis), {})
        instan = decomp(**inpars)
        result = instan.go()
        if outdir is not None:
            assert os.path.exists(outdir), f"Path {outdir} does not exist"
            instan.finalize(result, directory=outdir)
        return result

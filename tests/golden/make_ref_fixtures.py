"""Golden outputs of the reference 2LPT code itself, at small grids.

Builds the reference's own Aarambam/LPT/Basis and LPT/ResBasis sources
(compiled where they lie in the reference checkout, against the
single-process MPI / GSL-rng / FFTW2 stand-ins in oracle/shim, recipe
`make -C oracle ref`), runs the resulting executables on a few small
configurations and stores what they
writes -- the Gaussian and non-Gaussian potential dumps (write_phi) and the
Gadget snapshot -- as compressed .npz fixtures under tests/golden/ref/.

Inputs are synthetic: a BBKS transfer table, regular-lattice glass files,
and coefficient tables made by the reference Decomposer
(tests/golden/make_alpha_tables.py).

Usage: python tests/golden/make_ref_fixtures.py   (needs the reference checkout)
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from aarambam_gb300 import gadget, tables  # noqa: E402

OUT = os.path.join(HERE, "ref")

BASE = dict(Omega=0.3, OmegaLambda=0.7, OmegaBaryon=0.0, OmegaDM_2ndSpecies=0.0, HubbleParam=0.7,
            ShapeGamma=0.0, Sigma8=0.8, PrimordialIndex=0.965, Redshift=49.0, FixedAmplitude=0, PhaseFlip=0,
            SphereMode=0, SavePotentialField=1, WhichSpectrum=0, WhichTransfer=2,
            FileWithInputSpectrum="ThisIsAFakeStringThatIsNeverUsed", NumFilesWrittenInParallel=1,
            InputSpectrum_UnitLength_in_cm=3.085678e24, UnitLength_in_cm=3.085678e24, UnitMass_in_g=1.989e43,
            UnitVelocity_in_cm_per_s=1e5, WDM_On=0, WDM_Vtherm_On=0, WDM_PartMass_in_kev=10.0,
            FileBase="ics")

# name -> overrides; "table" names a directory under tests/golden/tables, glass = (n, tile)
CASES = {
    "local_n32": dict(Nmesh=32, Nsample=32, Nmax=128, Box=500.0, Seed=1234, Fnl=10.0, N_modes=8,
                      table="local_m8_L500_n128", glass=(16, 2)),
    "scalarI_n32_flip_fixed_cut": dict(Nmesh=32, Nsample=24, Nmax=256, Box=500.0, Seed=4321, Fnl=100.0,
                                       N_modes=10, PhaseFlip=1, FixedAmplitude=1,
                                       table="scalarI_m10_L500_n256", glass=(8, 4)),
    "scalarI12_n16_sphere": dict(Nmesh=16, Nsample=12, Nmax=512, Box=1000.0, Seed=7, Fnl=100.0, N_modes=12,
                                 SphereMode=1, table="scalarI_m12_L1000_n512", glass=(16, 1)),
    "local_n24": dict(Nmesh=24, Nsample=24, Nmax=128, Box=500.0, Seed=99, Fnl=-50.0, N_modes=8,
                      table="local_m8_L500_n128", glass=(12, 2)),
    # 2LPTResBasis (oscillating P(k)), one case per WhichSpectrum
    "res_lin_n32": dict(exe="2LPTResBasis", Nmesh=32, Nsample=32, Nmax=128, Box=500.0, Seed=31, Fnl=10.0,
                        N_modes=8, WhichSpectrum=1, A_res=0.5, w_res=30.0, phi_res=0.3,
                        table="local_m8_L500_n128", glass=(16, 2)),
    "res_log_n32": dict(exe="2LPTResBasis", Nmesh=32, Nsample=28, Nmax=256, Box=500.0, Seed=32, Fnl=100.0,
                        N_modes=10, WhichSpectrum=2, A_res=0.3, w_res=10.0, phi_res=0.0, PhaseFlip=1,
                        table="scalarI_m10_L500_n256", glass=(8, 4)),
    "res_both_n16": dict(exe="2LPTResBasis", Nmesh=16, Nsample=16, Nmax=512, Box=1000.0, Seed=33, Fnl=100.0,
                         N_modes=12, WhichSpectrum=0, A_res=0.9, w_res=2.0, phi_res=0.0, SphereMode=1,
                         table="scalarI_m12_L1000_n512", glass=(16, 1)),
}


def write_config(path, cfg):
    with open(path, "w") as f:
        for k, v in cfg.items():
            f.write(f"{k:<36s}{v}\n")


def run_case(name, spec, tmp):
    d = os.path.join(tmp, name)
    os.makedirs(d)
    k, t = tables.bbks_transfer()
    tables.write_transfer(os.path.join(d, "T.dat"), k, t)
    gn, tile = spec["glass"]
    gadget.write_glass(os.path.join(d, "glass.dat"), gadget.lattice_glass(gn, 100.0), 100.0)
    tdir = os.path.join(HERE, "tables", spec["table"])
    cfg = dict(BASE)
    cfg.update({kk: vv for kk, vv in spec.items() if kk not in ("table", "glass", "exe")})
    cfg.update(GlassFile=os.path.join(d, "glass.dat"), GlassTileFac=tile, OutputDir=d,
               FileWithInputTransfer=os.path.join(d, "T.dat"),
               FileWithAlphaCoeff=os.path.join(tdir, "AlphaTable.dat"),
               FileWithX0Coeff=os.path.join(tdir, "AiTable.dat"))
    write_config(os.path.join(d, "cfg"), cfg)
    exe = os.path.join(ROOT, "oracle", "_ref", spec.get("exe", "2LPTBasis"))
    res = subprocess.run([exe, os.path.join(d, "cfg")], capture_output=True, text=True, cwd=d)
    if res.returncode != 0:
        raise RuntimeError(res.stdout + res.stderr)
    seed = cfg["Seed"]
    pg, n, box = gadget.read_potential(os.path.join(d, f"Gauss_potential_{seed}"))
    pn, _, _ = gadget.read_potential(os.path.join(d, f"Nongauss_potential_{seed}"))
    h, pos, vel, ids = gadget.read_snapshot(os.path.join(d, "ics"))
    keep = {kk: vv for kk, vv in cfg.items() if kk not in ("GlassFile", "OutputDir", "FileWithInputTransfer",
                                                          "FileWithAlphaCoeff", "FileWithX0Coeff")}
    keep.update(table=spec["table"], glass_n=gn, glass_box=100.0)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), pot_gauss=pg, pot_ng=pn, pos=pos, vel=vel, ids=ids,
                        header=np.frombuffer(h.tobytes(), dtype=np.uint8), config=json.dumps(keep),
                        stdout=res.stdout)
    print(name, "ok", pos.shape)


if __name__ == "__main__":
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    os.makedirs(OUT, exist_ok=True)
    names = sys.argv[1:] or list(CASES)
    with tempfile.TemporaryDirectory() as tmp:
        for nm in names:
            run_case(nm, CASES[nm], tmp)

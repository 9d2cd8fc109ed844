"""`Aarambam-2LPT-Basis <paramfile>` and `Aarambam-2LPT-ResBasis <paramfile>`:
the reference executables' command lines (Aarambam/LPT/Basis/cli.py:5-10 and
LPT/ResBasis/cli.py:5-10 -> main.c:53-102) on one GPU.  ResBasis reads three
more tags (A_res, w_res, phi_res) and takes WhichSpectrum 0, 1 or 2 as its
P(k) oscillation mode.

Reads the same parameter file, coefficient tables, transfer table and glass,
runs the path through libaarambam_gpu.so and writes the same files:
  OutputDir/FileBase                     Gadget-1 snapshot (save.c:162-520)
  OutputDir/Gauss_potential_<Seed>       if SavePotentialField == 1
  OutputDir/Nongauss_potential_<Seed>    (write_phi, save.c:14-105)
  OutputDir/inputspec_<FileBase>.txt     (print_spec, main.c:1631-1694)
As in the reference, a missing argument or a bad parameter file prints the
reference's messages and exits with status 0.  One process writes one
snapshot file (the reference's single-task naming); the rank count given to
mpirun is irrelevant.
"""
from __future__ import annotations

import math
import os
import sys
import time

import numpy as np

from . import gadget, params, tables

PI = 3.14159265358979323846
GRAVITY = 6.672e-8
HUBBLE = 3.2407789e-18


class Transfer:
    """Tabulated transfer function (power.c:66-153, :181-217)."""

    def __init__(self, k, t, kconv):
        order = np.argsort(np.log10(k), kind="stable")
        self.logk = np.log10(k)[order]
        lt = np.log10(t)[order]
        self.logT = lt - lt[0]
        self.kconv = kconv

    def __call__(self, k: float) -> float:
        k = k * self.kconv
        if k <= 0:
            return 0.0
        lk = math.log10(k)
        L = self.logk
        if lk < L[0] or lk > L[-1]:
            return 0.0
        hi = int(np.searchsorted(L, lk, side="right"))
        hi = min(max(hi, 1), len(L) - 1)
        lo = hi - 1
        u = (lk - L[lo]) / (L[hi] - L[lo])
        return 10.0 ** ((1 - u) * self.logT[lo] + u * self.logT[hi])


def _growth(a, om, ol):
    from scipy.integrate import quad
    ha = math.sqrt(om / a ** 3 + (1 - om - ol) / a ** 2 + ol)
    return ha * quad(lambda x: (x / (om + (1 - om - ol) * x + ol * x ** 3)) ** 1.5, 0, a, epsabs=0,
                     epsrel=1e-10, limit=200)[0]


def power_osc(cfg, k):
    """The P(k) oscillation of 2LPTResBasis (ResBasis/power.c:240-260); 1 for
    a Basis parameter set."""
    if "A_res" not in cfg:
        return 1.0
    if cfg["WhichSpectrum"] == 1:
        return 1 + cfg["A_res"] * math.cos(cfg["w_res"] * k + cfg["phi_res"])
    if cfg["WhichSpectrum"] == 2:
        return 1 + cfg["A_res"] * math.cos(cfg["w_res"] * math.log(k) + cfg["phi_res"])
    return 1.0


def print_spec(path, cfg, norm, transfer):
    """inputspec_<FileBase>.txt (main.c:1631-1694): k, Delta^2, k_nl, Delta^2_nl
    (Peacock & Dodds)."""
    om, ol = cfg["Omega"], cfg["OmegaLambda"]
    ul = cfg["UnitLength_in_cm"]
    gf = _growth(1.0, om, ol) / _growth(0.001, om, ol) / (1.0 / 0.001)
    ddd = _growth(1.0, om, ol) / _growth(1.0 / (cfg["Redshift"] + 1), om, ol)

    def pk(k):
        t = transfer(k)
        return norm * math.exp(cfg["PrimordialIndex"] * math.log(k)) * power_osc(cfg, k) * t * t

    lines = [f"{cfg['Redshift']:12g} {ddd:12g}"]
    k = 2 * PI / (1000.0 * (3.085678e24 / ul))
    kend = 2 * PI / (0.001 * (3.085678e24 / ul))
    while k < kend:
        po = pk(k)
        dl = 4.0 * PI * k * k * k * po
        kf = 0.5
        po2, po1 = pk(1.001 * k * kf), pk(k * kf)
        knl = dnl = 0.0
        if po != 0 and po1 != 0 and po2 != 0:
            neff = (math.log(po2) - math.log(po1)) / (math.log(1.001 * k * kf) - math.log(k * kf))
            if 1 + neff / 3 > 0:
                A = 0.482 * (1 + neff / 3) ** -0.947
                B = 0.226 * (1 + neff / 3) ** -1.778
                alpha = 3.310 * (1 + neff / 3) ** -0.244
                beta = 0.862 * (1 + neff / 3) ** -0.287
                V = 11.55 * (1 + neff / 3) ** -0.423 * 1.2
                x = dl
                dnl = x * ((1 + B * beta * x + (A * x) ** (alpha * beta)) /
                           (1 + ((A * x) ** alpha * gf ** 3 / (V * math.sqrt(x))) ** beta)) ** (1 / beta)
                knl = k * (1 + dnl) ** (1.0 / 3)
        lines.append(f"{k:12g} {dl:12g}    {knl:12g} {dnl:12g}")
        k *= 1.025
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def snapshot_header(cfg, npart, init_time):
    """Gadget header the reference writes for one task (save.c:184-266)."""
    ul, um, uv = cfg["UnitLength_in_cm"], cfg["UnitMass_in_g"], cfg["UnitVelocity_in_cm_per_s"]
    ut = ul / uv
    G = GRAVITY / ul ** 3 * um * ut ** 2
    H = HUBBLE * ut
    m1 = cfg["Omega"] * 3 * H * H / (8 * PI * G) * cfg["Box"] ** 3 / npart
    return gadget.make_header(
        npart=[0, npart & 0xFFFFFFFF, 0, 0, 0, 0],
        npartTotal=[0, npart & 0xFFFFFFFF, (npart >> 32) & 0xFFFFFFFF, 0, 0, 0],
        mass=[0, m1, 0, 0, 0, 0], time=init_time, redshift=1.0 / init_time - 1, num_files=1,
        BoxSize=cfg["Box"], Omega0=cfg["Omega"], OmegaLambda=cfg["OmegaLambda"], HubbleParam=cfg["HubbleParam"])


def run(cfg: dict, precision: str = "fp32", log=print) -> dict:
    """One IC realisation for a parsed parameter-file dict; writes the files."""
    import torch

    from .ic import ICGenerator

    if cfg["WhichTransfer"] != 2:
        raise ValueError("only a tabulated transfer function (WhichTransfer 2) is supported")
    if "A_res" in cfg:
        if cfg["WhichSpectrum"] not in (0, 1, 2):
            raise ValueError("2LPTResBasis: WhichSpectrum must be 0, 1 or 2")
    elif cfg["WhichSpectrum"] != 0:
        raise ValueError("2LPTBasis: only WhichSpectrum 0 (the tabulated transfer function) is supported")
    if cfg["WDM_On"]:
        raise ValueError("WDM_On is not supported")
    M = cfg["N_modes"]
    alpha = tables.load_alpha(cfg["FileWithAlphaCoeff"], M)
    x0 = tables.load_x0(cfg["FileWithX0Coeff"], M)
    k, t = tables.load_transfer(cfg["FileWithInputTransfer"])
    glass, gh = gadget.read_glass(cfg["GlassFile"])
    tile = cfg["GlassTileFac"]
    t0 = time.time()
    gen = ICGenerator(cfg, alpha, x0, k, t, precision=precision)
    sc = gen.scalars
    N = cfg["Nmesh"]
    out = {}
    dev = gen.device
    g = torch.from_numpy(glass).to(dev)
    save = cfg["SavePotentialField"] == 1 and precision == "fp32"
    if save:
        gen.stage("noise")
        out["gauss"] = gen.c2r(gen.spectrum()).double().cpu().numpy()
        gen.stage("modal")
        out["nongauss"] = gen.c2r(gen.spectrum()).double().cpu().numpy()
        gen.stage("lpt")
        pos, vel, ids = gen.readout_glass(g, float(gh["BoxSize"]), tile)
    else:
        pos, vel, ids = gen.run_glass(g, float(gh["BoxSize"]), tile)
    torch.cuda.synchronize()
    pos, vel, ids = pos.cpu().numpy(), vel.cpu().numpy(), ids.cpu().numpy()
    log(f"path done in {time.time() - t0:.2f} s ({len(ids)} particles, {gen.launches} kernel launches)")
    od, fb, seed = cfg["OutputDir"], cfg["FileBase"], cfg["Seed"]
    if save:
        gadget.write_potential(os.path.join(od, f"Gauss_potential_{seed}"), out["gauss"], cfg["Box"])
        gadget.write_potential(os.path.join(od, f"Nongauss_potential_{seed}"), out["nongauss"], cfg["Box"])
    hdr = snapshot_header(cfg, len(ids), sc["init_time"])
    gadget.write_snapshot(os.path.join(od, fb), hdr, pos, vel, ids)
    kconv = cfg["InputSpectrum_UnitLength_in_cm"] / cfg["UnitLength_in_cm"]
    print_spec(os.path.join(od, f"inputspec_{fb}.txt"), cfg, sc["norm"], Transfer(k, t, kconv))
    return dict(pos=pos, vel=vel, ids=ids, scalars=sc, **out)


def main(argv=None, variant: str = "basis") -> int:
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        sys.stdout.write("\nParameters are missing.\nCall with <ParameterFile>\n\n")
        return 0
    sys.stdout.write("RUNNING LPTPNG WITH 1 TASKS")
    try:
        cfg = params.read_parameterfile(argv[0], variant)
    except params.ParameterError as e:
        for m in e.messages:
            sys.stdout.write(m + "\n")
        return 0
    precision = os.environ.get("AARAMBAM_PRECISION", "fp32")
    run(cfg, precision=precision, log=lambda s: sys.stdout.write("\n" + s + "\n"))
    return 0


def main_resbasis(argv=None) -> int:
    """`Aarambam-2LPT-ResBasis <paramfile>`."""
    return main(argv, "resbasis")


if __name__ == "__main__":
    # python -m aarambam_gb300.cli [--resbasis] <paramfile>
    if sys.argv[1:2] == ["--resbasis"]:
        sys.exit(main_resbasis(sys.argv[2:]))
    sys.exit(main())

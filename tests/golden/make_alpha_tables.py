"""Generate the alpha / X0 coefficient tables used as fixtures by the tests and the bench.

The tables are produced by the reference project's own Decomposer
(Aarambam/utils.py:349-446 -> Aarambam/basis/decompose.py:84-216), built from
its sources in a scratch directory (the Cython module Aarambam/basis/cmbbest.pyx
plus tetrapyd.c / arrays.c, compiled with gcc -fopenmp).  Nothing of the
reference is copied into this repository: only the two text tables each run
writes (AlphaTable.dat "p q r alpha", AiTable.dat "p x0 x1",
Aarambam/basis/decompose.py:297-321) are kept, under tests/golden/tables/<name>/.

Usage:  python tests/golden/make_alpha_tables.py [name ...]
Needs the reference checkout at /root/reference (read-only; it is copied).
"""
import json
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile
import time

import numpy as np

REF = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "tables")

# name -> (model class, n_modes, n_s, Lbox, Nmax, ModeTol, MaxModeCount, model kwargs)
CONFIGS = {
    # 128^3 plain-method case: Local template, 8 modes.  Nmax is raised from 64
    # to 128 because the 2LPT code asserts Nmax >= Nsample (main.c:200).
    "local_m8_L500_n128": ("Local", 8, 0.965, 500.0, 128, 1e-4, 150, {}),
    # 512^3 precision case: ScalarI mass=1, 12 modes.
    "scalarI_m12_L1000_n512": ("ScalarI", 12, 0.965, 1000.0, 512, 1e-4, 150, {"mass": 1.0}),
    # 256^3 adjoint case: ScalarI mass=1, 10 modes.
    "scalarI_m10_L500_n256": ("ScalarI", 10, 0.965, 500.0, 256, 1e-4, 150, {"mass": 1.0}),
    # small cases for the batch (templates and uneven mode counts at 256^3)
    "local_m6_L500_n256": ("Local", 6, 0.965, 500.0, 256, 1e-4, 150, {}),
    "equil_m9_L500_n256": ("Equilateral", 9, 0.965, 500.0, 256, 1e-4, 150, {}),
    "scalarI_m13_L500_n256_mu0p5": ("ScalarI", 13, 0.965, 500.0, 256, 1e-4, 150, {"mass": 0.5}),
    "scalarI_m16_L500_n256_mu1p5": ("ScalarI", 16, 0.965, 500.0, 256, 1e-4, 150, {"mass": 1.5}),
    # the batch's 20-mode template (mode counts 6..20 across the batch)
    "scalarI_m20_L500_n256_mu1p75": ("ScalarI", 20, 0.965, 500.0, 256, 1e-4, 150, {"mass": 1.75}),
    # 1024^3 headline: ScalarI mass=1, 20 modes, Box 1000.
    "scalarI_m20_L1000_n1024": ("ScalarI", 20, 0.965, 1000.0, 1024, 1e-4, 150, {"mass": 1.0}),
    # 1536^3 resonant case: LogResonance w=10, 20 modes, Box 2000.
    "logres_w10_m20_L2000_n1536": ("LogResonance", 20, 0.965, 2000.0, 1536, 1e-4, 150,
                                   {"w_res": 10.0, "phi": 0.0}),
}


def build_reference(tmp):
    src = os.path.join(REF, "Aarambam")
    dst = os.path.join(tmp, "Aarambam")
    shutil.copytree(src, dst)
    bdir = os.path.join(dst, "basis")
    subprocess.check_call(["cython", "-3", "cmbbest.pyx", "-o", "cmbbest.c"], cwd=bdir)
    inc = sysconfig.get_paths()["include"]
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-I" + inc,
                           "-I" + np.get_include(), "cmbbest.c", "tetrapyd.c", "arrays.c",
                           "-o", "cmbbest" + ext], cwd=bdir)
    return tmp


def run(name, tmp):
    model, m, ns, lbox, nmax, tol, maxc, kw = CONFIGS[name]
    os.environ.setdefault("TMPDIR", tmp)
    sys.path.insert(0, tmp)
    import Aarambam as Am  # noqa: E402  (the scratch copy)
    outdir = os.path.join(OUT, name)
    os.makedirs(outdir, exist_ok=True)
    t0 = time.time()
    dec = Am.utils.Decomposer(N_modes=m, n_s=ns, Lbox=lbox, Nmax=nmax, ModeTol=tol, MaxModeCount=maxc)
    # Aarambam.models exports SingleField and Colliders; the resonance
    # templates live in Aarambam.models.Resonances
    import Aarambam.models.Resonances as Res  # noqa: E402
    cls = getattr(Am.models, model, None) or getattr(Res, model)
    res = dec.go(cls, Am.basis.BasicBasisDecompose, outdir=outdir, **kw)
    dt = time.time() - t0
    tab = np.loadtxt(os.path.join(outdir, "AlphaTable.dat"))
    meta = dict(model=model, N_modes=m, n_s=ns, Lbox=lbox, Nmax=nmax, ModeTol=tol, MaxModeCount=maxc,
                model_kwargs=kw, seconds=round(dt, 1), nonzero_alpha=int(np.count_nonzero(tab[:, 3])),
                rows=int(tab.shape[0]))
    with open(os.path.join(outdir, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, meta, flush=True)


if __name__ == "__main__":
    names = sys.argv[1:] or list(CONFIGS)
    with tempfile.TemporaryDirectory() as tmp:
        build_reference(tmp)
        for n in names:
            run(n, tmp)

"""Configuration and post-processing helpers (reference Aarambam/utils.py)."""
import os
import struct

import numpy as np

from aarambam_gb300 import gadget, params, utils


def test_make_config_basis_parses_back(tmp_path):
    d = str(tmp_path)
    kw = dict(utils.DEFAULT_BASIS_INPUTS)
    kw.update(Nmesh=64, Nsample=64, Nmax=128, Lbox=500.0, OutputDir=d, seed=7, Fnl=12.5, N_modes=8,
              SavePotentialField=False, NWriteoutProcesses=2)
    path = os.path.join(d, "LPTconfig")
    with open(path, "w") as f:
        f.write(utils.make_config_basis(**kw))
    cfg = params.read_parameterfile(path)
    assert (cfg["Nmesh"], cfg["Nsample"], cfg["Nmax"], cfg["Seed"], cfg["N_modes"]) == (64, 64, 128, 7, 8)
    assert cfg["Box"] == 500.0 and cfg["Fnl"] == 12.5 and cfg["SavePotentialField"] == 0
    assert cfg["OutputDir"] == d and cfg["GlassFile"] == kw["GlassFile"]
    assert cfg["WhichSpectrum"] == 0 and cfg["WhichTransfer"] == 2 and cfg["NumFilesWrittenInParallel"] == 2


def test_make_example_config_basis_is_complete(tmp_path):
    path = os.path.join(str(tmp_path), "cfg")
    with open(path, "w") as f:
        f.write(utils.make_example_config_basis())
    cfg = params.read_parameterfile(path)
    assert cfg["Nmesh"] == 256 and cfg["GlassTileFac"] == 4 and cfg["SavePotentialField"] == 1


def test_collate_single_file_dumps(tmp_path):
    d = str(tmp_path)
    rng = np.random.default_rng(3)
    g, ng = rng.standard_normal((2, 8, 8, 8))
    gadget.write_potential(os.path.join(d, "Gauss_potential_42"), g, 100.0)
    gadget.write_potential(os.path.join(d, "Nongauss_potential_42"), ng, 100.0)
    out = utils.collate_potential(d)
    assert np.array_equal(out["Gauss_potential"], g) and np.array_equal(out["Nongauss_potential"], ng)
    assert not os.path.exists(os.path.join(d, "Gauss_potential_42"))


def write_slab(fname, field, x0, nx, box):
    """One rank's dump as write_phi writes it with several ranks (save.c:64-98)."""
    n = field.shape[1]
    with open(fname, "wb") as f:
        f.write(struct.pack("<iid", 0, n, box))
        for i in range(nx):
            for j in range(n):
                for k in range(n):
                    f.write(struct.pack("<id", (i * n + j) * (2 * (n // 2 + 1)) + k, field[x0 + i, j, k]))


def test_collate_slab_dumps(tmp_path):
    d = str(tmp_path)
    rng = np.random.default_rng(4)
    for t in ["Gauss_potential", "Nongauss_potential"]:
        f = rng.standard_normal((6, 6, 6))
        for x0, nx in [(0, 2), (2, 2), (4, 2)]:
            write_slab(os.path.join(d, f"{t}_9_StartX_{x0:04d}_NumX_{nx}"), f, x0, nx, 50.0)
        out = utils.collate_potential(d)
        assert np.array_equal(out[t], f)


def test_camb2input_columns(tmp_path):
    p = os.path.join(str(tmp_path), "camb.dat")
    a = np.arange(21, dtype=float).reshape(3, 7)
    np.savetxt(p, a)
    assert np.array_equal(utils.camb2input(p), a[:, [0, 6]])

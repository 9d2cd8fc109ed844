"""The Aarambam-2LPT-Basis command line: argument / parameter-file handling
(CPU) and its files against the reference executable's own (GPU)."""
import os

import numpy as np
import pytest

from aarambam_gb300 import cli, gadget, tables
from tests.common import GOLDEN, load_case, periodic_delta, rel_rms


def test_missing_argument_prints_usage_and_exits_zero(capsys):
    assert cli.main([]) == 0
    assert "Parameters are missing." in capsys.readouterr().out


def test_bad_parameter_file_exits_zero_with_messages(tmp_path, capsys):
    p = tmp_path / "cfg"
    p.write_text("Nmesh 32\nNmesh 64\n")
    assert cli.main([str(p)]) == 0
    out = capsys.readouterr().out
    assert "Tag 'Nmesh' not allowed or multiple defined." in out
    assert "I miss a value for tag 'Box'" in out


def write_case(tmp_path, name, save=1):
    cfg, z = load_case(name)
    d = str(tmp_path)
    k, t = tables.bbks_transfer()
    tables.write_transfer(os.path.join(d, "T.dat"), k, t)
    gadget.write_glass(os.path.join(d, "glass.dat"), gadget.lattice_glass(cfg["glass_n"], 100.0), 100.0)
    tdir = os.path.join(GOLDEN, "tables", cfg["table"])
    c = {k_: v for k_, v in cfg.items() if k_ not in ("table", "glass_n", "glass_box")}
    c.update(SavePotentialField=save, GlassFile=f"{d}/glass.dat", OutputDir=d, FileWithInputTransfer=f"{d}/T.dat",
             FileWithAlphaCoeff=f"{tdir}/AlphaTable.dat", FileWithX0Coeff=f"{tdir}/AiTable.dat")
    path = os.path.join(d, "cfg")
    with open(path, "w") as f:
        f.write("".join(f"{k_:<36s}{v}\n" for k_, v in c.items()))
    return path, cfg, z


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["local_n32", "scalarI_n32_flip_fixed_cut"])
def test_cli_files_match_reference(cuda, tmp_path, name):
    path, cfg, z = write_case(tmp_path, name)
    assert cli.main([path]) == 0
    d = str(tmp_path)
    h, pos, vel, ids = gadget.read_snapshot(os.path.join(d, cfg["FileBase"]))
    ref_h = np.frombuffer(z["header"].tobytes(), dtype=gadget.HEADER_DTYPE)[0]
    for f in ("npart", "npartTotal", "num_files"):
        assert np.array_equal(h[f], ref_h[f]), f
    for f in ("mass", "time", "redshift", "BoxSize", "Omega0", "OmegaLambda", "HubbleParam"):
        assert np.allclose(h[f], ref_h[f], rtol=1e-9, atol=0), f
    assert np.array_equal(ids, z["ids"])
    glass = gadget.lattice_glass(cfg["glass_n"], 100.0)
    from oracle import oracle as O
    o = O.Oracle(cfg, *tables.bbks_transfer())
    lagr = o.tile_glass(glass, 100.0, cfg["GlassTileFac"])
    assert rel_rms(periodic_delta(pos, lagr, cfg["Box"]), periodic_delta(z["pos"], lagr, cfg["Box"])) < 1e-5
    assert rel_rms(vel, z["vel"]) < 1e-5
    pg, n, box = gadget.read_potential(os.path.join(d, f"Gauss_potential_{cfg['Seed']}"))
    pn, _, _ = gadget.read_potential(os.path.join(d, f"Nongauss_potential_{cfg['Seed']}"))
    assert n == cfg["Nmesh"] and box == cfg["Box"]
    assert rel_rms(pg, z["pot_gauss"]) < 1e-6
    assert rel_rms(pn, z["pot_ng"]) < 1e-6
    spec = np.loadtxt(os.path.join(d, f"inputspec_{cfg['FileBase']}.txt"), skiprows=1)
    assert spec.shape[1] == 4 and np.all(np.isfinite(spec))

"""2LPTResBasis: the oscillating primordial spectrum (Aarambam/LPT/ResBasis).

The same path with P(k) times (1 + A_res cos(w_res k + phi_res)) and/or
(1 + A_res cos(w_res ln k + phi_res)) by WhichSpectrum: in the sigma8
normalisation (ResBasis/power.c:240-260) and on the Gaussian potential's
per-cell power, where the switch falls through (ResBasis/main.c:445-455).
Checked against the reference ResBasis executable's own outputs
(tests/golden/ref/res_*.npz) and the FP64 oracle."""
import os

import numpy as np
import pytest
import torch

from aarambam_gb300 import _lib, cli, gadget, params, utils
from tests.common import RES_CASES, bbks, lattice_lagrangian, load_case, make_cfg, periodic_delta, rel_rms, table


def res_cfg(N, mode, **kw):
    c = make_cfg(N, 500.0, 77 + mode, 50.0, 8, "local_m8_L500_n128", 128, **kw)
    c.update(WhichSpectrum=mode, A_res=0.6, w_res=25.0 if mode == 1 else 8.0, phi_res=0.4)
    return c


# ------------------------------------------------------------ CPU
def test_resbasis_tag_table():
    assert len(params.TAGS_RESBASIS) == len(params.TAGS) + 3
    names = [t for t, _ in params.TAGS_RESBASIS]
    i = names.index("SavePotentialField")
    assert names[i + 1:i + 4] == ["A_res", "w_res", "phi_res"]
    basis_text = utils.make_example_config_basis()
    with pytest.raises(params.ParameterError) as e:
        params.parse_parameter_text(basis_text, "f", "resbasis")
    assert "Error. I miss a value for tag 'A_res' in parameter file 'f'." in e.value.messages


def test_resbasis_config_text_round_trip():
    cfg = params.parse_parameter_text(utils.make_config_resbasis(**dict(utils.DEFAULT_RESBASIS_INPUTS, Pk_mode=2,
                                                                        Pk_A_res=0.25, Pk_w_res=7.5,
                                                                        Pk_phi_res=0.1)), "f", "resbasis")
    assert (cfg["WhichSpectrum"], cfg["A_res"], cfg["w_res"], cfg["phi_res"]) == (2, 0.25, 7.5, 0.1)


def test_resbasis_cli_usage(capsys):
    assert cli.main_resbasis([]) == 0
    assert "Parameters are missing." in capsys.readouterr().out


def test_resbasis_params_reach_the_abi():
    from aarambam_gb300.ic import params_from_config
    p = params_from_config(res_cfg(32, 2))
    assert (p.variant, p.which_spectrum, p.a_res, p.w_res, p.phi_res) == (_lib.AAR_VARIANT_RESBASIS, 2, 0.6, 8.0,
                                                                        0.4)
    q = params_from_config(make_cfg(32, 500.0, 1, 10.0, 8, "t", 128))
    assert (q.variant, q.which_spectrum) == (_lib.AAR_VARIANT_BASIS, 0)


# ------------------------------------------------------------ GPU
def gen_for(cfg, precision="fp32"):
    from aarambam_gb300.ic import ICGenerator
    return ICGenerator(cfg, *table(cfg["table"], cfg["N_modes"]), *bbks(), precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("name", RES_CASES)
def test_resbasis_particles_vs_reference_outputs(cuda, name):
    from oracle import oracle as O
    cfg, z = load_case(name)
    g = gen_for(cfg)
    o = O.Oracle(cfg, *bbks())
    assert abs(g.scalars["norm"] / o.scalars["Norm"] - 1) < 1e-9
    lagr = lattice_lagrangian(o, cfg["glass_n"], cfg["GlassTileFac"])
    pos, vel = g.run(torch.from_numpy(lagr).cuda())
    d_gpu = periodic_delta(pos.cpu().numpy(), lagr, cfg["Box"])
    d_ref = periodic_delta(z["pos"], lagr, cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-5
    assert rel_rms(vel.cpu().numpy(), z["vel"]) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_resbasis_gaussian_spectrum_vs_oracle(cuda, mode):
    from oracle import oracle as O
    cfg = res_cfg(64, mode)
    g = gen_for(cfg)
    g.stage("noise")
    got = g.spectrum().cpu().numpy()
    ref = O.Oracle(cfg, *bbks()).gauss()
    ref = ref[..., 0] + 1j * ref[..., 1]
    assert np.array_equal(got != 0, ref != 0)
    nz = ref != 0
    assert (np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])).max() < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_resbasis_plain_fp64_vs_oracle(cuda, mode):
    """The plain FP64 form evaluates the oscillation per cell in the noise
    kernel (the reference's formula): particles to FP64 rounding."""
    from oracle import oracle as O
    cfg = res_cfg(32, mode)
    o = O.Oracle(cfg, *bbks())
    lagr = lattice_lagrangian(o, 32, 1)
    r = o.run(*table(cfg["table"], cfg["N_modes"]), lagr)
    pos, vel = gen_for(cfg, precision="fp64").run(torch.from_numpy(lagr).cuda())
    d_gpu = periodic_delta(pos.cpu().numpy(), lagr, cfg["Box"])
    d_ref = periodic_delta(r["pos"], lagr, cfg["Box"])
    assert rel_rms(d_gpu, d_ref) < 1e-6
    assert rel_rms(vel.cpu().numpy(), r["vel"]) < 1e-6


@pytest.mark.gpu
def test_resbasis_cli_files_match_reference(cuda, tmp_path):
    cfg, z = load_case("res_lin_n32")
    d = str(tmp_path)
    k, t = bbks()
    from aarambam_gb300 import tables
    tables.write_transfer(os.path.join(d, "T.dat"), k, t)
    gadget.write_glass(os.path.join(d, "glass.dat"), gadget.lattice_glass(cfg["glass_n"], 100.0), 100.0)
    from tests.common import GOLDEN
    tdir = os.path.join(GOLDEN, "tables", cfg["table"])
    c = {k_: v for k_, v in cfg.items() if k_ not in ("table", "glass_n", "glass_box")}
    c.update(SavePotentialField=1, GlassFile=f"{d}/glass.dat", OutputDir=d, FileWithInputTransfer=f"{d}/T.dat",
             FileWithAlphaCoeff=f"{tdir}/AlphaTable.dat", FileWithX0Coeff=f"{tdir}/AiTable.dat")
    path = os.path.join(d, "cfg")
    with open(path, "w") as f:
        f.write("".join(f"{k_:<36s}{v}\n" for k_, v in c.items()))
    assert cli.main_resbasis([path]) == 0
    pg, n, box = gadget.read_potential(os.path.join(d, f"Gauss_potential_{cfg['Seed']}"))
    pn, _, _ = gadget.read_potential(os.path.join(d, f"Nongauss_potential_{cfg['Seed']}"))
    assert rel_rms(pg, z["pot_gauss"]) < 1e-6
    assert rel_rms(pn, z["pot_ng"]) < 1e-6
    h, pos, vel, ids = gadget.read_snapshot(os.path.join(d, cfg["FileBase"]))
    assert rel_rms(vel, z["vel"]) < 1e-5

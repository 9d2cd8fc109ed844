"""Host-side logic: parameter file, tables, Gadget I/O, the C ABI's exports
and the arithmetic of the RANLUX skip-ahead (all on CPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from aarambam_gb300 import _lib, gadget, params, tables
from aarambam_gb300.build import LIB, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CONFIG = """
Nmesh                               32
Nsample                             32
Nmax                                128
Box                                 500.000000
FileBase                            ics
OutputDir                           /tmp/x
GlassFile                           /tmp/x/glass.dat
GlassTileFac                        2

Seed                                1234
% a comment line
Omega                               0.300000
OmegaLambda                         0.700000
OmegaBaryon                         0.00000 #Doesn't really matter
OmegaDM_2ndSpecies                  0.00
HubbleParam                         0.700000
Sigma8                              0.800000
PrimordialIndex                     0.965000
Redshift                            49.000000
Fnl                                 10.000000
N_modes                             8
FixedAmplitude                      0
PhaseFlip                           0
SphereMode                          0
SavePotentialField                  0
WhichSpectrum                       0 #Fixed
WhichTransfer                       2 #Fixed
FileWithInputSpectrum               ThisIsAFakeStringThatIsNeverUsed
FileWithInputTransfer               /tmp/x/T.dat
FileWithAlphaCoeff                  /tmp/x/AlphaTable.dat
FileWithX0Coeff                     /tmp/x/AiTable.dat
NumFilesWrittenInParallel           1
InputSpectrum_UnitLength_in_cm      3.085678e24 #One Mpc in cm
UnitLength_in_cm                    3.085678e24
UnitMass_in_g                       1.989e43
UnitVelocity_in_cm_per_s            1e5
ShapeGamma                          0.0
WDM_On                              0
WDM_Vtherm_On                       0
WDM_PartMass_in_kev                 10.0
"""


def test_parameter_file_parses_every_tag():
    v = params.parse_parameter_text(CONFIG)
    assert set(v) == {t for t, _ in params.TAGS}
    assert v["Nmesh"] == 32 and v["Box"] == 500.0 and v["UnitLength_in_cm"] == 3.085678e24
    assert v["FileWithInputSpectrum"] == "ThisIsAFakeStringThatIsNeverUsed"


def test_parameter_file_missing_and_duplicate_tags():
    bad = CONFIG.replace("Sigma8                              0.800000\n", "")
    bad += "Nmesh 64\nBogusTag 1\n"
    with pytest.raises(params.ParameterError) as e:
        params.parse_parameter_text(bad, "cfg")
    msgs = e.value.messages
    assert "Error in file cfg:   Tag 'Nmesh' not allowed or multiple defined." in msgs
    assert "Error in file cfg:   Tag 'BogusTag' not allowed or multiple defined." in msgs
    assert "Error. I miss a value for tag 'Sigma8' in parameter file 'cfg'." in msgs


def test_c_number_conversions():
    assert params.c_atoi("42abc") == 42 and params.c_atoi("x") == 0 and params.c_atoi("-7") == -7
    assert params.c_atof("1e5") == 1e5 and params.c_atof("3.5foo") == 3.5 and params.c_atof("bar") == 0.0


def test_missing_parameter_file():
    with pytest.raises(params.ParameterError, match="not found"):
        params.read_parameterfile("/nonexistent/cfg")


def test_alpha_table_is_symmetrised(tmp_path):
    p = tmp_path / "A.dat"
    p.write_text(" 3 1 0 2.5 \n 2 2 1 -1e-11 \n 1 1 1 0.5\n")
    a = tables.load_alpha(str(p), 4)
    for perm in [(3, 1, 0), (3, 0, 1), (1, 3, 0), (1, 0, 3), (0, 3, 1), (0, 1, 3)]:
        assert a[perm] == 2.5
    assert a[1, 2, 2] == -1e-11 and a[1, 1, 1] == 0.5
    assert np.count_nonzero(a) == 6 + 3 + 1


def test_alpha_table_errors(tmp_path):
    p = tmp_path / "A.dat"
    p.write_text("9 0 0 1.0\n")
    with pytest.raises(tables.TableError):
        tables.load_alpha(str(p), 4)
    with pytest.raises(tables.TableError):
        tables.load_alpha(str(tmp_path / "missing"), 4)


def test_x0_and_transfer(tmp_path):
    p = tmp_path / "Ai.dat"
    p.write_text(" 0 1 0 \n 1 -1.0073643243302743 0 \n")
    x0 = tables.load_x0(str(p), 3)
    assert x0[0] == 1 and x0[1] == -1.0073643243302743 and x0[2] == 0
    k, t = tables.bbks_transfer()
    tables.write_transfer(str(tmp_path / "T.dat"), k, t)
    k2, t2 = tables.load_transfer(str(tmp_path / "T.dat"))
    assert np.allclose(k, k2, rtol=1e-15) and np.allclose(t, t2, rtol=1e-15)


def test_active_pairs_match_fixture_counts():
    from tests.common import table
    a, _ = table("scalarI_m12_L1000_n512", 12)
    pairs = tables.active_pairs(a)
    assert len(pairs) == 59  # the reference transforms 59 (N_i, N_j) pairs for this table


def test_glass_and_snapshot_round_trip(tmp_path):
    g = gadget.lattice_glass(8, 100.0)
    gadget.write_glass(str(tmp_path / "g.dat"), g, 100.0)
    pos, h = gadget.read_glass(str(tmp_path / "g.dat"))
    assert np.array_equal(pos, g) and h["BoxSize"] == 100.0 and h["npartTotal"][1] == 512
    hdr = gadget.make_header(npart=[0, 512, 0, 0, 0, 0], BoxSize=100.0, num_files=1)
    ids = np.arange(1, 513, dtype=np.int32)
    gadget.write_snapshot(str(tmp_path / "s"), hdr, g, g * 0.5, ids)
    h2, p2, v2, i2 = gadget.read_snapshot(str(tmp_path / "s"))
    assert np.array_equal(p2, g) and np.array_equal(v2, g * 0.5) and np.array_equal(i2, ids)
    assert os.path.getsize(str(tmp_path / "s")) == (8 + 256) + 2 * (8 + 12 * 512) + (8 + 4 * 512)


def test_truncated_glass_is_rejected(tmp_path):
    g = gadget.lattice_glass(4, 100.0)
    gadget.write_glass(str(tmp_path / "g.dat"), g, 100.0)
    data = open(tmp_path / "g.dat", "rb").read()
    open(tmp_path / "t.dat", "wb").write(data[:-20])
    with pytest.raises(gadget.GadgetError):
        gadget.read_glass(str(tmp_path / "t.dat"))


def test_potential_dump_layout(tmp_path):
    f = np.arange(4 ** 3, dtype=np.float64).reshape(4, 4, 4)
    gadget.write_potential(str(tmp_path / "pot"), f, 500.0)
    g, n, box = gadget.read_potential(str(tmp_path / "pot"))
    assert n == 4 and box == 500.0 and np.array_equal(g, f)
    rec = np.memmap(str(tmp_path / "pot"), offset=16, dtype=gadget.POT_DTYPE, mode="r")
    assert rec["coord"][5] == (0 * 4 + 1) * 2 * 3 + 1  # (i*N + j) * 2(N/2+1) + k


def test_params_struct_mirrors_header():
    """The ctypes aar_params has the header's fields, in order, with the same
    C types (the plan reads the caller's struct by layout)."""
    hdr = open(os.path.join(ROOT, "include", "aarambam.h")).read()
    body = re.search(r"typedef struct aar_params \{(.*?)\} aar_params;", hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), ctype) for n in names.split(",")]
    ct = {"int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "double": ctypes.c_double}
    assert [(n, ct[t]) for n, t in fields] == list(_lib.Params._fields_)


def test_c_abi_library_exports_every_declared_symbol():
    build()
    hdr = open(os.path.join(ROOT, "include", "aarambam.h")).read()
    declared = set(re.findall(r"^\s*(?:int|int64_t|void|size_t|const char\*)\s+(aar_[A-Za-z0-9_]+)\s*\(", hdr, re.M))
    assert declared == set(_lib.EXPORTS)
    L = ctypes.CDLL(LIB)
    for name in declared:
        assert hasattr(L, name), name
    assert L.aar_version() == 1


# ---- arithmetic behind the seed-table skip-ahead (ranlux.cuh) ----
B = 1 << 48
MOD = B ** 12 - B ** 5 + 1


def _seed_words(sd):
    v = sd & 0xFFFFFFFF
    bits = [(v >> k) & 1 for k in range(31)]
    ib, jb, xs = 0, 18, []
    for _ in range(12):
        w = 0
        for _ in range(48):
            w = 2 * w + (bits[ib] ^ 1)
            bits[ib] ^= bits[jb]
            ib, jb = (ib + 1) % 31, (jb + 1) % 31
        xs.append(w)
    return xs


def test_skip_ahead_window_integer():
    seq = _seed_words(98765)
    car = [0] * 12
    c = 0
    for n in range(12, 12 + 3000):
        d = seq[n - 5] - seq[n - 12] - c
        c = int(d < 0)
        seq.append(d + B if d < 0 else d)
        car.append(c)

    def K(t):
        P = sum(seq[t + n] * B ** n for n in range(12))
        Q = sum(seq[t + n] * B ** n for n in range(7))
        return P - B ** 5 * Q - car[t + 11] * B ** 12

    binv = pow(B, -1, MOD)
    assert (B * (B ** 11 - B ** 4) + 1) % MOD == 0          # b^-1 = -(b^11 - b^4)
    for t in (13, 202, 404, 2020):
        assert -MOD <= K(t) <= 0
        r = (K(0) * pow(binv, t, MOD)) % MOD
        V = MOD - r
        digs = []
        for _ in range(13):
            d = (-V) % B
            digs.append(d)
            V = (V + MOD * d) // B
        assert digs[:12] == seq[t:t + 12]
        assert (digs[7] - digs[0] - digs[12]) % B == car[t + 11]


def test_multi_file_glass(tmp_path):
    """A glass split over files base.0, base.1 (find_files, read_glass.c:226-260)."""
    rng = np.random.default_rng(2)
    a = rng.uniform(0, 100, (40, 3)).astype(np.float32)
    b = rng.uniform(0, 100, (24, 3)).astype(np.float32)
    base = str(tmp_path / "glass")
    for i, part in enumerate((a, b)):
        h = gadget.make_header(npart=[0, len(part), 0, 0, 0, 0], npartTotal=[0, 64, 0, 0, 0, 0], num_files=2,
                               BoxSize=100.0)
        with open(f"{base}.{i}", "wb") as f:
            gadget._write_record(f, h.tobytes())
            gadget._write_record(f, part.astype("<f4").tobytes())
    assert gadget.glass_files(base) == [f"{base}.0", f"{base}.1"]
    pos, h = gadget.read_glass(base)
    assert np.array_equal(pos, np.concatenate([a, b])) and int(h["num_files"]) == 2

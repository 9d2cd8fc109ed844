"""The CPU oracle against known answers and the reference's own outputs."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.common import CASES, RES_CASES, bbks, lattice_lagrangian, load_case, rel_rms, table


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()


def test_ranlxd_known_answers():
    # GSL's published known-answer values: seed 1, 10000th gsl_rng_get
    r1 = O.Ranlux(1, 202)
    for _ in range(9999):
        r1.get()
    assert r1.get() == 1998227290
    r2 = O.Ranlux(1, 397)
    for _ in range(9999):
        r2.get()
    assert r2.get() == 3949287736


def test_ranlux_seed_zero_is_seed_one():
    a, b = O.Ranlux(0), O.Ranlux(1)
    assert [a.get() for _ in range(50)] == [b.get() for _ in range(50)]


@pytest.mark.parametrize("N", [8, 16, 24, 32])
def test_fft_matches_numpy(N):
    rng = np.random.default_rng(N)
    x = rng.standard_normal((N, N, N))
    c = O.r2c(x)
    ref = np.fft.rfftn(x)
    assert np.abs(c[..., 0] + 1j * c[..., 1] - ref).max() < 1e-10 * np.abs(ref).max()
    # c2r of a NON-Hermitian half spectrum: FFTW drops what breaks symmetry in
    # the kz = 0 and kz = N/2 planes (numpy's irfftn has the same semantics)
    X = rng.standard_normal((N, N, N // 2 + 1)) + 1j * rng.standard_normal((N, N, N // 2 + 1))
    y = O.c2r(np.stack([X.real, X.imag], -1))
    yr = np.fft.irfftn(X, s=(N, N, N), axes=(0, 1, 2)) * N**3
    assert np.abs(y - yr).max() < 1e-10 * np.abs(yr).max()


def test_seedtable_shell_order_is_a_permutation():
    for N in (4, 16, 24, 64):
        pos = []
        for i in range(N // 2):
            pos += [i * N + j for j in range(i)] + [j * N + i for j in range(i + 1)]
            pos += [(N - 1 - i) * N + j for j in range(i)] + [(N - 1 - j) * N + i for j in range(i + 1)]
            pos += [i * N + (N - 1 - j) for j in range(i)] + [j * N + (N - 1 - i) for j in range(i + 1)]
            pos += [(N - 1 - i) * N + (N - 1 - j) for j in range(i)]
            pos += [(N - 1 - j) * N + (N - 1 - i) for j in range(i + 1)]
        assert sorted(pos) == list(range(N * N))


def test_seedtable_first_values():
    # the first draws of the Seed stream land at (0,0), then shell 1, ...
    o = O.Ranlux(1234)
    u = [o.uniform() for _ in range(5)]
    cfg, _ = load_case("local_n32")
    k, t = bbks()
    orc = O.Oracle(cfg, k, t)
    st = orc.seedtable()
    N = cfg["Nmesh"]
    # shell 0 fills the four corners, then shell 1 starts at (1, 0)
    for d, (i, j) in enumerate([(0, 0), (N - 1, 0), (0, N - 1), (N - 1, N - 1), (1, 0)]):
        assert st[i, j] == int(0x7FFFFFFF * u[d])


@pytest.mark.parametrize("name", CASES + RES_CASES)
def test_oracle_reproduces_reference_outputs(name):
    """Oracle vs the reference's own main.c/power.c/read_glass.c built on the
    single-process stand-ins (tests/golden/make_ref_fixtures.py)."""
    cfg, z = load_case(name)
    k, t = bbks()
    o = O.Oracle(cfg, k, t)
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    lagr = lattice_lagrangian(o, cfg["glass_n"], cfg["GlassTileFac"])
    r = o.run(alpha, x0, lagr)
    assert rel_rms(r["pot_gauss"], z["pot_gauss"]) < 1e-13
    assert rel_rms(r["pot_ng"], z["pot_ng"]) < 1e-12
    assert np.array_equal(r["pos"], z["pos"]) or np.abs(r["pos"] - z["pos"]).max() < 1e-4
    assert rel_rms(r["vel"], z["vel"]) < 1e-10
    assert np.array_equal(z["ids"], np.arange(1, len(z["ids"]) + 1))


def test_oracle_scalars_are_finite_and_reference_like():
    cfg, z = load_case("local_n32")
    k, t = bbks()
    s = O.Oracle(cfg, k, t).scalars
    assert all(np.isfinite(v) for v in s.values())
    # the reference prints "Normfac=%g" (power.c:418)
    out = str(z["stdout"])
    normfac = float(out.split("Normfac=")[1].split(")")[0])
    assert abs(s["Norm"] / normfac - 1) < 1e-5


def test_oracle_rejects_short_transfer_table():
    cfg, _ = load_case("local_n32")
    k = np.logspace(-3, 2, 50)
    with pytest.raises(RuntimeError, match="1111"):
        O.Oracle(cfg, k, np.ones_like(k))


@pytest.mark.parametrize("name", RES_CASES)
def test_resbasis_normalisation_and_oscillation(name):
    """ResBasis: sigma8 normalisation with the oscillating PowerSpec (the
    reference prints Normfac), and the fixtures do depend on the oscillation:
    the same run without it misses the reference's Gaussian potential."""
    cfg, z = load_case(name)
    k, t = bbks()
    s = O.Oracle(cfg, k, t).scalars
    normfac = float(str(z["stdout"]).split("Normfac=")[1].split(")")[0])
    assert abs(s["Norm"] / normfac - 1) < 1e-5
    plain = {kk: v for kk, v in cfg.items() if kk not in ("A_res", "w_res", "phi_res")}
    plain["WhichSpectrum"] = 0
    o = O.Oracle(plain, k, t)
    alpha, x0 = table(cfg["table"], cfg["N_modes"])
    r = o.run(alpha, x0, lattice_lagrangian(o, cfg["glass_n"], cfg["GlassTileFac"]))
    assert rel_rms(r["pot_gauss"], z["pot_gauss"]) > 1e-2

"""The CPU oracle (C restatement) against the reference's golden fixtures and physics
invariants.  No GPU needed."""
import numpy as np
import pytest

from cudaprob3_gb300 import earth
from oracle.oracle import Mixing as OMix, OracleError
from tests.conftest import golden_files
from tests.helpers import oracle_on_fixture, vacuum_probabilities

NOM = OMix(0.5843, 0.1496, 0.7365, -1.601, 7.53e-5, 2.49e-3, 1)


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_matches_reference_fixture(oracle, path):
    d = np.load(path)
    got = oracle_on_fixture(oracle, d)
    # Same arithmetic in the same order: bit-exact on the machine that made the fixtures;
    # a different libm / FMA use may move the last bits.
    np.testing.assert_allclose(got, d["out"], rtol=0, atol=1e-13)


def test_reference_probe_values(oracle):
    """Values of the reference's own build on the headline atmospheric grid."""
    r, rho, ye = earth.PREM_4LAYER
    cz, en = earth.cosine_grid(400), earth.log_energy_grid(400)
    out = oracle.atmos(NOM, False, cz[[0, 100]], en[[0, 200]], r, rho, ye, 22.0)
    assert abs(out[0, 0, 4] - 0.29218904109825022) < 1e-14
    assert abs(out[1, 1, 3] - 0.025924148531545836) < 1e-14
    b = oracle.beam(NOM, False, earth.lin_energy_grid(100000)[[5000]], 2.6, 1300.0)
    assert abs(b[0, 3] - 0.041147220859941214) < 1e-14


@pytest.mark.parametrize("model", ["prem4", "shells59", "poly"])
@pytest.mark.parametrize("anti", [False, True])
def test_unitarity(oracle, model, anti):
    rng = np.random.default_rng(3)
    mix = OMix(*rng.uniform(0.1, 1.4, 3), rng.uniform(-3, 3), 7.4e-5, -2.5e-3 if anti else 2.5e-3,
               -1 if anti else 1)
    cz, en = np.linspace(-1, 1, 31), np.logspace(-1, 2, 23)
    if model == "poly":
        r, a, b, c, ye = earth.PREM_4LAYER_QUAD_V2
        out = oracle.atmos(mix, anti, cz, en, r, None, ye, 15.0, poly_abc=(a, b, c))
    else:
        r, rho, ye = earth.PREM_4LAYER if model == "prem4" else earth.synthetic_shells(59)
        out = oracle.atmos(mix, anti, cz, en, r, rho, ye, 15.0)
    P = out.reshape(31, 23, 3, 3)
    np.testing.assert_allclose(P.sum(-1), 1.0, atol=1e-11)  # sum over final flavours
    np.testing.assert_allclose(P.sum(-2), 1.0, atol=1e-11)  # sum over initial flavours


@pytest.mark.parametrize("anti", [False, True])
def test_vacuum_limit_matches_analytic(oracle, anti):
    mix = OMix(0.59, 0.15, 0.78, 0.9, 7.4e-5, 2.5e-3, -1 if anti else 1)
    en = np.logspace(-1, 1.5, 40)
    b = oracle.beam(mix, anti, en, 0.0, 810.0)
    ref = vacuum_probabilities(mix, 810.0, en, antineutrino=anti)
    np.testing.assert_allclose(b, ref, atol=1e-12)


def test_downgoing_is_vacuum_over_path_length(oracle):
    """cos >= 0: one air segment of the production-point-to-detector length."""
    r, rho, ye = earth.PREM_4LAYER
    cz = np.array([0.0, 0.3, 1.0])
    en = np.logspace(-1, 1, 11)
    out = oracle.atmos(NOM, False, cz, en, r, rho, ye, 22.0)
    R, h = 6371.0, 22.0
    for i, c in enumerate(cz):
        L = np.sqrt((R + h) ** 2 - R * R * (1 - c * c)) - R * c
        np.testing.assert_allclose(out[i], vacuum_probabilities(NOM, L, en), atol=1e-12)


def test_time_reversal_symmetric_profile(oracle):
    """The Earth profile is palindromic, so P(a->b; dcp) = P(b->a; -dcp)."""
    r, rho, ye = earth.PREM_4LAYER
    cz, en = np.linspace(-1, -0.1, 9), np.logspace(-1, 1.5, 9)
    m1 = OMix(0.58, 0.15, 0.74, 1.1, 7.5e-5, 2.5e-3, 1)
    m2 = OMix(0.58, 0.15, 0.74, -1.1, 7.5e-5, 2.5e-3, 1)
    p1 = oracle.atmos(m1, False, cz, en, r, rho, ye, 0.0).reshape(9, 9, 3, 3)
    p2 = oracle.atmos(m2, False, cz, en, r, rho, ye, 0.0).reshape(9, 9, 3, 3)
    np.testing.assert_allclose(p1, np.swapaxes(p2, -1, -2), atol=1e-11)


def test_max_layers_and_limit(oracle):
    r = earth.PREM_4LAYER[0][::-1].copy()
    lim = -np.sqrt(1 - r ** 2 / 6371.0 ** 2)
    lim[0] = 0.0
    cz = np.array([1.0, 0.0, -1e-9, lim[1] + 1e-9, lim[1] - 1e-9, -1.0])
    m, rc = oracle.max_layers(r, cz)
    assert rc == 0
    assert list(m) == [0, 0, 1, 1, 2, 5 - 1]
    m, rc = oracle.max_layers(r, np.array([-1.0]), limit=3)
    assert rc == 3  # "setMaxlayers : invalid number of maxLayer"


def test_model_order_checks(oracle):
    with pytest.raises(OracleError, match="order"):
        oracle.flip_model(np.array([0.0, 3000.0, 2000.0, 6371.0]), np.ones(4))
    rd, rho = oracle.flip_model(np.array([0.0, 1.0, 2.0]), np.array([5.0, 6.0, 7.0]))
    assert list(rd) == [2.0, 1.0, 0.0] and list(rho) == [7.0, 6.0, 5.0]
    rd2, _ = oracle.flip_model(rd, rho)
    assert list(rd2) == [2.0, 1.0, 0.0]  # already descending: unchanged


def test_trajectory_lengths_add_up(oracle):
    """Segments of an up-going trajectory sum (in and out) to the full path length."""
    r, rho, ye = earth.PREM_4LAYER
    for c in (-0.95, -0.6, -0.2):
        L, dens = oracle.trajectory(r, rho, ye, c, 22.0)
        total = L[0] + 2 * L[1:-1].sum() + L[-1]
        R, h = 6371.0, 22.0
        path = np.sqrt((R + h) ** 2 - R * R * (1 - c * c)) - R * c
        assert abs(total - path) < 1e-9
        assert dens[0] == 0.0

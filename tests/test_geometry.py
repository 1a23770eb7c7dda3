"""Host-side trajectory geometry of the C ABI (cp3_trajectory_table, no GPU) against the
oracle's restatement of getTraversedDistanceOfLayer / getDensityOfLayer[Poly]: bit-exact,
including shell-grazing and out-of-range cosines."""
import numpy as np
import pytest

from cudaprob3_gb300 import _abi, earth
from tests.conftest import golden_files


@pytest.fixture(scope="module", autouse=True)
def built():
    from cudaprob3_gb300 import build
    build.build()


def compare(oracle, radii, rho, ye, cosines, h, poly_abc=None):
    if poly_abc is None:
        t = _abi.trajectory_table(radii, rho, ye, cosines, h)
    else:
        t = _abi.trajectory_table(radii, poly_abc[0], ye, cosines, h, c2=poly_abc[1],
                                  c3=poly_abc[2], poly=True)
    for ic, c in enumerate(cosines):
        L, dens = oracle.trajectory(radii, rho, ye, c, h, poly_abc=poly_abc)
        a, b = t["seg_offset"][ic], t["seg_offset"][ic + 1]
        assert b - a == len(L)
        np.testing.assert_array_equal(t["seg_len_km"][a:b], L)
        np.testing.assert_array_equal(t["seg_rho_e"][a:b], dens)
    return t


@pytest.mark.parametrize("path", [f for f in golden_files("atmos")],
                         ids=lambda p: p.split("/")[-1][:-4])
def test_fixture_geometry_bit_exact(oracle, path):
    d = np.load(path)
    poly = (d["a"], d["b"], d["c"]) if int(d["poly"]) else None
    compare(oracle, d["radii"], d["rho"], d["ye"], d["cosines"], float(d["h_km"]), poly)


def test_classes_and_random_cosines(oracle):
    r, rho, ye = earth.synthetic_shells(59)
    cz = np.sort(np.random.default_rng(1).uniform(-1, 1, 500))
    t = compare(oracle, r, rho, ye, cz, 22.0)
    rd, rhod, yed = r[::-1], rho[::-1], ye[::-1]
    assert t["class_rho_e"][0] == 0.0
    np.testing.assert_array_equal(t["class_rho_e"][1:], (rhod * yed)[:len(t["class_rho_e"]) - 1])
    seg_rho = t["seg_rho_e"]
    np.testing.assert_array_equal(seg_rho, t["class_rho_e"][t["seg_class"]])


def test_layer_limit_reported():
    r = np.linspace(0, 6371, 200)
    with pytest.raises(_abi.CP3Error, match="invalid number of maxLayer"):
        _abi.trajectory_table(r, np.ones(200), np.full(200, 0.5), [-1.0], 10.0)

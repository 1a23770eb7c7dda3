"""Production-height averaging (physics.hpp:997-1067, switched on explicitly: the
reference's own switch never enables it) on the FP64 and mixed kernels, against the fixture
made by the reference's calculate_atmos and against the oracle."""
import os

import numpy as np
import pytest

from cudaprob3_gb300 import AtmosCudaPropagatorSingle, earth
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def run_avg(prec, mix6, knu, anti, cz, en, radii, rho, ye, h, nb, prob, edges, poly_abc=None):
    p = AtmosCudaPropagatorSingle(0, len(cz), len(en), precision=prec)
    p.setEnergyList(en)
    p.setCosineList(cz)
    p.setMNSMatrix(*mix6[:4], knu)
    p.setNeutrinoMasses(mix6[4], mix6[5])
    if poly_abc is None:
        p.setDensity(radii, rho, ye)
    else:
        p.setDensity(radii, *poly_abc, ye)
    p.setProductionHeight(h)
    p.SetNumberOfProductionHeightBinsForAveraging(nb)
    p.setProductionHeightList(prob, edges)
    p.calculateProbabilities(1 if anti else 0)
    return p.probabilities()


def test_averaging_matches_reference_fixture():
    d = np.load(os.path.join(GOLDEN, "atmos_avg.npz"))
    for t, knu in ((0, 1), (1, -1)):
        got = run_avg("fp64", d["mix"], knu, t == 1, d["cosines"], d["energies"], d["radii"],
                      d["rho"], d["ye"], float(d["h_km"]), int(d["avg_bins"]), d["avg_prob"],
                      d["avg_edges"])
        assert np.abs(got - d["out"][t]).max() <= 1e-12


@pytest.mark.parametrize("poly", [False, True])
def test_averaging_against_oracle(oracle, poly):
    from oracle.oracle import Mixing as OMix
    rng = np.random.default_rng(2)
    cz, en = np.linspace(-1, 1, 33), earth.log_energy_grid(29)
    nb = 5
    w = rng.uniform(0.2, 1.0, (2, 3, len(en), len(cz), nb))
    w /= w.sum(axis=-1, keepdims=True)
    edges = np.array([8.0, 12.0, 17.0, 24.0, 33.0, 45.0])
    m = earth.gaussian_sets(1, seed=40)[0]
    mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    if poly:
        r, a, b, c, ye = earth.PREM_4LAYER_QUAD_V2
        rho, abc = None, (a, b, c)
    else:
        r, rho, ye = earth.PREM_4LAYER
        abc = None
    for anti, knu in ((False, 1), (True, -1)):
        ref = oracle.atmos(OMix(*mix6[:4], mix6[4], mix6[5], knu), anti, cz, en, r, rho, ye, 20.0,
                           poly_abc=abc, avg=(nb, w.ravel(), edges))
        got = run_avg("fp64", mix6, knu, anti, cz, en, r, rho, ye, 20.0, nb, w.ravel(), edges, abc)
        assert np.abs(got - ref).max() <= 1e-12


def test_mixed_averaging_matches_reference_fixture():
    d = np.load(os.path.join(GOLDEN, "atmos_avg.npz"))
    for t, knu in ((0, 1), (1, -1)):
        got = run_avg("mixed", d["mix"], knu, t == 1, d["cosines"], d["energies"], d["radii"],
                      d["rho"], d["ye"], float(d["h_km"]), int(d["avg_bins"]), d["avg_prob"],
                      d["avg_edges"])
        assert np.abs(got - d["out"][t]).max() <= 1e-5


@pytest.mark.parametrize("shells", [4, 59])
def test_mixed_averaging_against_oracle(oracle, shells):
    """Wide production-height bins (the shift phases reach hundreds of rad at low energy) on
    4 and 59 shells, both neutrino types, all nine channels."""
    from oracle.oracle import Mixing as OMix
    rng = np.random.default_rng(3)
    cz, en = np.linspace(-1, 1, 41), earth.log_energy_grid(37)
    nb = 8
    w = rng.uniform(0.1, 1.0, (2, 3, len(en), len(cz), nb))
    w /= w.sum(axis=-1, keepdims=True)
    edges = np.linspace(2.0, 60.0, nb + 1)
    m = earth.gaussian_sets(1, seed=41)[0]
    mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    r, rho, ye = earth.PREM_4LAYER if shells == 4 else earth.synthetic_shells(59)
    for anti, knu in ((False, 1), (True, -1)):
        ref = oracle.atmos(OMix(*mix6[:4], mix6[4], mix6[5], knu), anti, cz, en, r, rho, ye, 20.0,
                           avg=(nb, w.ravel(), edges))
        got = run_avg("mixed", mix6, knu, anti, cz, en, r, rho, ye, 20.0, nb, w.ravel(), edges)
        assert np.abs(got - ref).max() <= 1e-5


@pytest.mark.parametrize("scale", [1.0, 1.15])
def test_mixed_averaging_with_quadratic_density_against_oracle(oracle, scale):
    """Averaging and the quadratic density model together on the mixed kernels (the
    reference runs them in one loop: physics.hpp:997-1067 with getDensityOfLayerPoly,
    physics.hpp:651-739): per-segment eigen-solves, the air layer's eigencomponents and the
    shift factors, against the oracle, both neutrino types, all nine channels, <= 1e-5.  The
    quadratic PREM, and the same profile 15 % denser."""
    from oracle.oracle import Mixing as OMix
    rng = np.random.default_rng(5)
    cz, en = np.linspace(-1, 1, 37), earth.log_energy_grid(31)
    nb = 6
    w = rng.uniform(0.1, 1.0, (2, 3, len(en), len(cz), nb))
    w /= w.sum(axis=-1, keepdims=True)
    edges = np.linspace(3.0, 50.0, nb + 1)
    m = earth.gaussian_sets(2, seed=43)[1]
    mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    r, a, b, c, ye = earth.PREM_4LAYER_QUAD_V2
    a, b, c = a * scale, b * scale, c * scale
    for anti, knu in ((False, 1), (True, -1)):
        ref = oracle.atmos(OMix(*mix6[:4], mix6[4], mix6[5], knu), anti, cz, en, r, None, ye, 20.0,
                           poly_abc=(a, b, c), avg=(nb, w.ravel(), edges))
        got = run_avg("mixed", mix6, knu, anti, cz, en, r, None, ye, 20.0, nb, w.ravel(), edges,
                      (a, b, c))
        assert np.abs(got - ref).max() <= 1e-5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("poly", [False, True])
def test_averaged_results_to_host_in_row_pieces(prec, poly):
    """calculate_to_host_async with averaging on: every averaging kernel (FP64, mixed, and
    the quadratic-density forms) runs in row pieces whose copies overlap the next piece, and
    the host buffer equals the device result for any number of pieces."""
    import torch
    nc, ne, nb = 41, 37, 5
    m = earth.NOMINAL
    edges = np.linspace(5.0, 45.0, nb + 1)
    prob = np.full((2, 3, ne, nc, nb), 1.0 / nb)
    p = AtmosCudaPropagatorSingle(0, nc, ne, precision=prec)
    p.setEnergyList(earth.log_energy_grid(ne))
    p.setCosineList(earth.cosine_grid(nc))
    p.setMNSMatrix(m.theta12, m.theta13, m.theta23, m.dcp, 1)
    p.setNeutrinoMasses(m.dm12sq, m.dm23sq)
    if poly:
        p.setDensity(*earth.PREM_4LAYER_QUAD_V2)
    else:
        p.setDensity(*earth.PREM_4LAYER)
    p.setProductionHeight(22.0)
    p.SetNumberOfProductionHeightBinsForAveraging(nb)
    p.setProductionHeightList(prob.ravel(), edges)
    p.calculateProbabilities(0)
    want = p.result().copy()
    dtype = torch.float64 if prec == "fp64" else torch.float32
    for chunks in (1, 3, 7, nc):
        host = torch.full((9 * nc * ne,), -1.0, dtype=dtype, pin_memory=True)
        p.calculate_to_host_async(0, host.data_ptr(), chunks)
        p.synchronize()
        assert np.array_equal(host.numpy().reshape(want.shape), want), chunks

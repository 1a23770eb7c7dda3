"""CUDA path (through the C ABI) against the reference's golden fixtures and the CPU oracle.

Tolerances (max absolute error per probability, every channel):
  FP64 kernels   <= 1e-12  (the drop-in bar)
  mixed kernels  <= 1e-5   (FP32 matrix work, FP64 eigen-decomposition, double-float phase)
Fixtures with exactly degenerate vacuum masses (the reference's 5e-9 eV^2 degeneracy break)
are ill-conditioned by construction: the reference's own result moves by ~1e-11 under
one-ulp changes of its transcendental functions, so FP64 parity there is checked to 1e-9.
"""
import os

import numpy as np
import pytest

from tests.conftest import golden_files
from tests.gpu_helpers import run_atmos, run_beam, run_fixture

pytestmark = pytest.mark.gpu

GPU_FIXTURES = [f for f in golden_files() if "avg" not in os.path.basename(f)]
FP64_TOL = 1e-12
MIXED_TOL = 1e-5
DEGENERATE_TOL = 1e-9


def _fp64_tol(path):
    return DEGENERATE_TOL if "deg" in os.path.basename(path) else FP64_TOL


@pytest.mark.parametrize("path", GPU_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_fp64_matches_reference_fixture(path):
    d = np.load(path)
    got = run_fixture(d, "fp64")
    err = np.abs(got - d["out"]).max()
    assert err <= _fp64_tol(path), err


@pytest.mark.parametrize("path", GPU_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_mixed_matches_reference_fixture(path):
    d = np.load(path)
    got = run_fixture(d, "mixed")
    err = np.abs(got - d["out"]).max()
    assert err <= MIXED_TOL, err


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("anti", [False, True])
def test_59_shells_against_oracle(oracle, prec, tol, anti):
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    r, rho, ye = earth.synthetic_shells(59)
    cz, en = earth.cosine_grid(160), earth.log_energy_grid(96)
    m = earth.NOMINAL
    knu = -1 if anti else 1
    ref = oracle.atmos(OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu),
                       anti, cz, en, r, rho, ye, 22.0)
    got = run_atmos(prec, [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq], knu,
                    anti, cz, en, r, rho, ye, 22.0)
    assert np.abs(got - ref).max() <= tol


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_the_largest_earth_model_against_oracle(oracle, prec, tol):
    """128 shells, the most a trajectory may cross (CP3_MAX_SHELLS): the vertical up-going
    rows cross every one, 257 layer applications of the reference's palindrome.  FP64 and
    mixed single propagators and one batched problem against the oracle; 129 shells are
    refused."""
    from cudaprob3_gb300 import earth
    from cudaprob3_gb300.batch import Batch
    from oracle.oracle import Mixing as OMix
    r, rho, ye = earth.synthetic_shells(128)
    cz = np.array([-1.0, -0.9999, -0.99, -0.7, -0.2, 0.0, 0.6])
    en = earth.log_energy_grid(48)
    m = earth.gaussian_sets(3, seed=77)[2]
    mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    for anti, knu in ((False, 1), (True, -1)):
        ref = oracle.atmos(OMix(*mix6, knu), anti, cz, en, r, rho, ye, 15.0, layer_limit=128)
        got = run_atmos(prec, mix6, knu, anti, cz, en, r, rho, ye, 15.0)
        assert np.abs(got - ref).max() <= tol
        if prec == "mixed":
            b = Batch(0)
            b.set_earth(r, rho, ye, 15.0)
            pid = b.add_atmos(cz, en)
            b.set_params(pid, m, anti)
            b.commit()
            b.run()
            b.synchronize()
            assert np.abs(np.transpose(b.result(pid), (1, 2, 0)) - ref).max() <= tol
    r2, rho2, ye2 = earth.synthetic_shells(129)
    with pytest.raises(RuntimeError, match="invalid number of maxLayer"):
        run_atmos(prec, mix6, 1, False, cz, en, r2, rho2, ye2, 15.0)


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_random_parameters_against_oracle(oracle, prec, tol):
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    rng = np.random.default_rng(11)
    r, rho, ye = earth.PREM_12LAYER
    cz, en = np.sort(rng.uniform(-1, 1, 37)), np.sort(rng.uniform(0.1, 50, 45))
    for m in earth.gaussian_sets(6, seed=5):
        for anti, knu in ((False, 1), (True, -1)):
            ref = oracle.atmos(OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq,
                                    knu), anti, cz, en, r, rho, ye, 15.0)
            got = run_atmos(prec, [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq],
                            knu, anti, cz, en, r, rho, ye, 15.0)
            assert np.abs(got - ref).max() <= tol


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("L", [295.0, 1300.0])
def test_beam_against_oracle(oracle, prec, tol, L):
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    en = earth.lin_energy_grid(20000)
    for m in earth.gaussian_sets(4, seed=9):
        for anti, knu in ((False, 1), (True, -1)):
            ref = oracle.beam(OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq,
                                   knu), anti, en, 2.6, L)
            got = run_beam(prec, [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq],
                           knu, anti, en, 2.6, L)
            assert np.abs(got - ref).max() <= tol


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_quadratic_density_against_oracle(oracle, prec, tol):
    """getDensityOfLayerPoly model (physics.hpp:651-739): every segment its own density."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    r, a, b, c, ye = earth.PREM_4LAYER_QUAD_V2
    cz, en = np.linspace(-1, 1, 61), earth.log_energy_grid(47)
    for m in earth.gaussian_sets(3, seed=21):
        for anti, knu in ((False, 1), (True, -1)):
            ref = oracle.atmos(OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq,
                                    knu), anti, cz, en, r, None, ye, 18.0, poly_abc=(a, b, c))
            got = run_atmos(prec, [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq],
                            knu, anti, cz, en, r, None, ye, 18.0, poly_abc=(a, b, c))
            assert np.abs(got - ref).max() <= tol


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_tiny_grids_against_oracle(oracle, prec, tol):
    """One bin, one cosine row, one energy column, and a beam of one energy: every launch
    shape's edge (a partial warp, a single block, one table entry per class)."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    r, rho, ye = earth.PREM_4LAYER
    m = earth.NOMINAL
    cases = [(np.array([-1.0]), np.array([2.5])),
             (np.array([-0.6]), earth.log_energy_grid(300)),
             (np.linspace(-1, 1, 300), np.array([0.7])),
             (np.array([-0.9, 0.3]), np.array([0.3, 4.0, 40.0]))]
    for cz, en in cases:
        for anti, knu in ((False, 1), (True, -1)):
            om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
            mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
            ref = oracle.atmos(om, anti, cz, en, r, rho, ye, 22.0)
            got = run_atmos(prec, mix6, knu, anti, cz, en, r, rho, ye, 22.0)
            assert got.shape == ref.shape
            assert np.abs(got - ref).max() <= tol, (len(cz), len(en), anti)
            got_b = run_beam(prec, mix6, knu, anti, en[:1], 2.6, 1300.0)
            ref_b = oracle.beam(om, anti, en[:1], 2.6, 1300.0)
            assert np.abs(got_b - ref_b).max() <= tol


@pytest.mark.parametrize("prec,tol,lo", [("fp64", FP64_TOL, 0.05), ("mixed", MIXED_TOL, 0.01)])
def test_energies_far_outside_the_configurations(oracle, prec, tol, lo):
    """Energies from 0.01 GeV (phases of ~1e4 rad through the core; FP64 from 0.05 GeV, where
    the reference's own phase roundings stay below its 1e-12 bar) to 10 TeV, where the matter
    potential dwarfs the splittings and two levels sit within 1e-3 of the spread, so the mixed
    solver hands many entries to its FP64 fallback.  PREM-4 and PREM-12, both orderings."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    cz = np.linspace(-1, 1, 41)
    en = np.logspace(np.log10(lo), 4, 60)
    for model in (earth.PREM_4LAYER, earth.PREM_12LAYER):
        r, rho, ye = model
        for m in earth.gaussian_sets(256, seed=2024)[::127]:  # sets 0, 127 (normal), 254 (inverted)
            for anti, knu in ((False, 1), (True, -1)):
                mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
                ref = oracle.atmos(OMix(*mix6[:4], *mix6[4:], knu), anti, cz, en, r, rho, ye, 22.0)
                got = run_atmos(prec, mix6, knu, anti, cz, en, r, rho, ye, 22.0)
                assert np.abs(got - ref).max() <= tol, (len(r), m.dm23sq, anti)
            ref_b = oracle.beam(OMix(*mix6[:4], *mix6[4:], 1), False, en, 2.6, 1300.0)
            got_b = run_beam(prec, mix6, 1, False, en, 2.6, 1300.0)
            assert np.abs(got_b - ref_b).max() <= tol

"""The precision study at full size: 59 equal shells, 2000 cos x 2000 log-E (0.1-100 GeV),
neutrino and antineutrino.  FP64 kernel against the oracle on a slice of cosine rows
(<= 1e-12), then the mixed kernel against the FP64 kernel on every one of the 4e6 bins and
every channel (<= 1e-5, the mixed-precision bar)."""
import os

import numpy as np
import pytest

from cudaprob3_gb300 import earth
from tests.gpu_helpers import run_atmos

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("anti", [False, True])
def test_precision_study_59_shells_full_grid(oracle, anti):
    from oracle.oracle import Mixing as OMix
    m = earth.NOMINAL
    mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    knu = -1 if anti else 1
    r, rho, ye = earth.synthetic_shells(59)
    cz, en = earth.cosine_grid(2000), earth.log_energy_grid(2000)
    f64 = run_atmos("fp64", mix6, knu, anti, cz, en, r, rho, ye, 22.0)
    mixed = run_atmos("mixed", mix6, knu, anti, cz, en, r, rho, ye, 22.0)
    rows = np.concatenate([np.arange(0, 40), np.arange(40, 2000, 97)])  # all deep rows + a spread
    ref = oracle.atmos(OMix(*mix6[:4], mix6[4], mix6[5], knu), anti, cz[rows], en, r, rho, ye,
                       22.0, nthreads=os.cpu_count() or 1)
    assert np.abs(f64[rows] - ref).max() <= 1e-12
    err = np.abs(mixed - f64).max(axis=(0, 1))  # per channel
    assert err.max() <= 1e-5, err


def test_beam_mixed_within_1e5_over_baselines_densities_and_low_energies():
    """Beam mixed kernel against the FP64 kernel where the phases are largest: baselines up to
    the Earth's diameter, densities up to the core's, energies down to 0.05 GeV (phases past
    1e3 rad, many of them reduced to within rounding of a half-turn)."""
    from tests.gpu_helpers import run_beam
    en = np.geomspace(0.05, 100.0, 20000)
    worst = 0.0
    for i, m in enumerate(earth.gaussian_sets(4, seed=7)):
        for dm23 in (m.dm23sq, -abs(m.dm23sq)):
            mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, dm23]
            for L in (295.0, 1300.0, 5000.0, 12742.0):
                for rho in (2.6, 4.5, 13.0):
                    for anti in (False, True):
                        knu = -1 if anti else 1
                        f = run_beam("fp64", mix6, knu, anti, en, rho, L)
                        g = run_beam("mixed", mix6, knu, anti, en, rho, L)
                        worst = max(worst, float(np.abs(f - g).max()))
    assert worst <= 1e-5, worst


def test_atmospheric_mixed_within_1e5_over_models_heights_and_low_energies():
    """Atmospheric mixed kernels (table and quadratic-density) against the FP64 kernels over
    Earth models (PREM 4 and 12 layers, 59 shells, the quadratic PREM), production heights,
    both orderings, nu and nubar, and energies down to 0.05 GeV, below the configurations'
    0.1 GeV (the 59-shell grid's largest errors, ~9e-6, sit there on core-crossing rows)."""
    cz = earth.cosine_grid(200)
    en = np.geomspace(0.05, 100.0, 300)
    qr, qa, qb, qc, qy = earth.PREM_4LAYER_QUAD_V2
    models = [earth.PREM_4LAYER, earth.PREM_12LAYER, earth.synthetic_shells(59), None]
    worst = {}
    for mi, model in enumerate(models):
        for m in earth.gaussian_sets(2, seed=9):
            for dm23 in (m.dm23sq, -abs(m.dm23sq)):
                mix6 = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, dm23]
                for h in (0.0, 22.0, 100.0):
                    for anti in (False, True):
                        knu = -1 if anti else 1
                        if model is None:
                            args = (cz, en, qr, None, qy, h, (qa, qb, qc))
                        else:
                            args = (cz, en, *model, h)
                        f = run_atmos("fp64", mix6, knu, anti, *args)
                        g = run_atmos("mixed", mix6, knu, anti, *args)
                        worst[mi] = max(worst.get(mi, 0.0), float(np.abs(f - g).max()))
    assert max(worst.values()) <= 1e-5, worst


def test_mixed_on_degenerate_mixing_parameters():
    """Parameter sets where a state has no electron component (theta13 = 0, theta12 = 0,
    theta12 = pi/2) or a splitting nearly vanishes: the mixed eigen-solver's rank-one
    eigenvector formula has no content for the decoupled state there and must hand it to the
    FP64 reference path.  Mixed against FP64 (beam and atmospheric) within 1e-5, no NaN."""
    from tests.gpu_helpers import run_beam
    m = earth.NOMINAL
    base = [m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq]
    cases = []
    for name, idx, val in (("theta13=0", 1, 0.0), ("theta12=0", 0, 0.0),
                           ("theta12=pi/2", 0, np.pi / 2), ("dm21=1e-9", 4, 1e-9)):
        mix6 = list(base)
        mix6[idx] = val
        cases.append((name, mix6))
    en = np.geomspace(0.1, 100.0, 2000)
    cz, ena = earth.cosine_grid(100), earth.log_energy_grid(200)
    worst = {}
    for name, mix6 in cases:
        for dm23 in (mix6[5], -abs(mix6[5])):
            mx = mix6[:5] + [dm23]
            for anti in (False, True):
                knu = -1 if anti else 1
                for L in (1300.0, 12742.0):
                    f = run_beam("fp64", mx, knu, anti, en, 2.6, L)
                    g = run_beam("mixed", mx, knu, anti, en, 2.6, L)
                    worst[name] = max(worst.get(name, 0.0), float(np.abs(f - g).max()))
                f = run_atmos("fp64", mx, knu, anti, cz, ena, *earth.PREM_4LAYER, 22.0)
                g = run_atmos("mixed", mx, knu, anti, cz, ena, *earth.PREM_4LAYER, 22.0)
                worst[name] = max(worst.get(name, 0.0), float(np.abs(f - g).max()))
    assert all(v <= 1e-5 for v in worst.values()), worst

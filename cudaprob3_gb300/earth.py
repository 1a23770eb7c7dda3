"""Earth models, oscillation-parameter sets and grids used by the workloads.

Models are given the way the reference's ``AtmosCpuPropagator::setDensity`` takes them
(atmoscpupropagator.hpp:116-170): one row per radius, ascending from the r=0 row, with the
density of the shell that ends at that radius.  The PREM tables are the public
Dziewonski-Anderson (1981) PREM values as shipped in the reference's ``models/*.dat``.
"""
from __future__ import annotations

import numpy as np

from .types import Mixing

# models/PREM_4layer.dat: radius (km), density (g/cm^3), Z/A
PREM_4LAYER = (
    np.array([0.0, 1220.0, 3480.0, 5701.0, 6371.0]),
    np.array([13.0, 13.0, 11.3, 5.0, 3.3]),
    np.array([0.468, 0.468, 0.468, 0.497, 0.497]),
)

# models/PREM_12layer.dat (two columns: radius, density). The file carries no Z/A; the
# core rows (r <= 3480 km) get 0.468 and the mantle rows 0.497, as in PREM_4layer.dat.
_PREM12_R = np.array([0.00, 1221.50, 1974.33, 2727.17, 3480.00, 4220.33, 4960.67, 5701.00,
                      5971.00, 6346.60, 6356.00, 6368.00, 6371.00])
_PREM12_RHO = np.array([13.0, 13.0, 11.948163, 11.341572, 10.462371, 5.381883, 5.007959,
                        4.603493, 3.9, 3.4, 2.900000, 2.600000, 1.020000])
CORE_RADIUS_KM = 3480.0
YE_CORE = 0.468
YE_MANTLE = 0.497


def ye_rule(radii) -> np.ndarray:
    """Z/A per row: 0.468 for rows at or inside the core radius, 0.497 outside."""
    r = np.asarray(radii, dtype=np.float64)
    return np.where(r <= CORE_RADIUS_KM, YE_CORE, YE_MANTLE)


PREM_12LAYER = (_PREM12_R, _PREM12_RHO, ye_rule(_PREM12_R))

# models/PREM_4layer_quad_v2.dat: radius, a (g/cm^5), b (g/cm^4), c (g/cm^3), Z/A for
# rho(r) = a r^2 + b r + c with r in km.
PREM_4LAYER_QUAD_V2 = (
    np.array([0.0, 1221.5, 3480.0, 5701.0, 6371.0]),
    np.array([-2.1779e-7, -2.1779e-7, -2.46861e-7, -3.0796e-8, -1.72335e-6]),
    np.array([0.0, 0.0, 1.71088e-4, -2.4486e-4, 1.9358e-2]),
    np.array([13.09, 13.09, 12.31, 6.78, -50.42]),
    np.array([0.468, 0.468, 0.468, 0.497, 0.497]),
)


def synthetic_shells(n_shells: int = 59, seed: int = 1234, jitter: float = 0.01):
    """Equal-thickness shells to 6371 km with a seeded monotone density profile.

    13.1 g/cm^3 at the centre falling to 9.9 at the core-mantle boundary (3480 km), then
    5.6 falling to 2.6 at the surface; each shell gets a seeded +-``jitter`` relative
    perturbation, after which the profile is made monotone (non-increasing outwards) again.
    Returns (radii, rho, ye) with the r=0 row first.
    """
    rng = np.random.default_rng(seed)
    radii = 6371.0 * np.arange(n_shells + 1) / n_shells
    mid = 0.5 * (radii[:-1] + radii[1:])
    core = mid <= CORE_RADIUS_KM
    rho_shell = np.where(core,
                         13.1 + (9.9 - 13.1) * mid / CORE_RADIUS_KM,
                         5.6 + (2.6 - 5.6) * (mid - CORE_RADIUS_KM) / (6371.0 - CORE_RADIUS_KM))
    rho_shell = rho_shell * (1.0 + jitter * rng.uniform(-1.0, 1.0, n_shells))
    rho_shell = np.minimum.accumulate(rho_shell)  # monotone non-increasing outwards
    rho = np.concatenate([[rho_shell[0]], rho_shell])  # row i>0 carries shell (r_{i-1}, r_i]
    ye = np.where(np.concatenate([[True], core]), YE_CORE, YE_MANTLE)
    return radii, rho, ye


# Parameters of the headline atmospheric configuration (also the centre of the Gaussian
# parameter sets of the batched workloads).
NOMINAL = Mixing(theta12=0.5843, theta13=0.1496, theta23=0.7365, dcp=-1.601,
                 dm12sq=7.53e-5, dm23sq=2.49e-3)
PRODUCTION_HEIGHT_KM = 22.0


def cosine_grid(n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    return np.linspace(lo, hi, n)


def log_energy_grid(n: int, lo: float = 0.1, hi: float = 100.0) -> np.ndarray:
    return np.logspace(np.log10(lo), np.log10(hi), n)


def lin_energy_grid(n: int, lo: float = 0.1, hi: float = 10.0) -> np.ndarray:
    return np.linspace(lo, hi, n)


def gaussian_sets(n_sets: int, seed: int = 2024, centre: Mixing = NOMINAL,
                  inverted_from: int | None = None) -> list[Mixing]:
    """Seeded parameter sets around ``centre``: sigma 0.02 rad on the angles, 1.0 rad on dcp,
    3% on both mass splittings.  Sets with index >= ``inverted_from`` (default: the second
    half) use inverted ordering, dm23sq = -|dm23sq|."""
    rng = np.random.default_rng(seed)
    if inverted_from is None:
        inverted_from = n_sets // 2
    out = []
    for i in range(n_sets):
        t12, t13, t23 = (centre.theta12 + 0.02 * rng.standard_normal(),
                         centre.theta13 + 0.02 * rng.standard_normal(),
                         centre.theta23 + 0.02 * rng.standard_normal())
        dcp = centre.dcp + 1.0 * rng.standard_normal()
        dm12 = centre.dm12sq * (1.0 + 0.03 * rng.standard_normal())
        dm23 = centre.dm23sq * (1.0 + 0.03 * rng.standard_normal())
        if i >= inverted_from:
            dm23 = -abs(dm23)
        out.append(Mixing(t12, t13, t23, dcp, dm12, dm23))
    return out


def uneven_grids(n_sets: int, seed: int = 2025, cos_range=(100, 1000), e_range=(100, 2000)):
    """Per-set grid sizes (n_cos, n_E), each uniform on the inclusive ranges."""
    rng = np.random.default_rng(seed)
    nc = rng.integers(cos_range[0], cos_range[1] + 1, n_sets)
    ne = rng.integers(e_range[0], e_range[1] + 1, n_sets)
    return [(int(a), int(b)) for a, b in zip(nc, ne)]

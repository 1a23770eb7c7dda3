"""Shared test helpers: run a golden fixture's inputs through the oracle."""
import numpy as np

from oracle.oracle import Mixing as OMix


def fixture_mix(d, knutype):
    m = d["mix"]
    return OMix(float(m[0]), float(m[1]), float(m[2]), float(m[3]), float(m[4]), float(m[5]),
                knutype)


def oracle_on_fixture(oracle, d):
    outs = []
    for t, knu in ((0, 1), (1, -1)):
        mix = fixture_mix(d, knu)
        if str(d["kind"]) == "atmos":
            abc = (d["a"], d["b"], d["c"]) if int(d["poly"]) else None
            avg = ((int(d["avg_bins"]), d["avg_prob"], d["avg_edges"])
                   if "avg_bins" in d.files else None)
            outs.append(oracle.atmos(mix, t == 1, d["cosines"], d["energies"], d["radii"],
                                     d["rho"], d["ye"], float(d["h_km"]), poly_abc=abc, avg=avg))
        else:
            outs.append(oracle.beam(mix, t == 1, d["energies"], float(d["rho"]), float(d["L"])))
    return np.stack(outs)


def vacuum_probabilities(mix, L_km, E, antineutrino=False):
    """Independent 3-flavour vacuum formula: P(a->b) = |sum_k U_ak^* U_bk e^{-i m_k L/2E}|^2
    with the PDG matrix and phases 2.534 m_k L / E (same unit factor as the reference)."""
    s12, s13, s23 = np.sin([mix.theta12, mix.theta13, mix.theta23])
    c12, c13, c23 = np.cos([mix.theta12, mix.theta13, mix.theta23])
    d = -mix.dcp if antineutrino else mix.dcp
    e = np.exp(-1j * d)
    U = np.array([[c12 * c13, s12 * c13, s13 * e],
                  [-s12 * c23 - c12 * s23 * s13 / e, c12 * c23 - s12 * s23 * s13 / e, s23 * c13],
                  [s12 * s23 - c12 * c23 * s13 / e, -c12 * s23 - s12 * c23 * s13 / e, c23 * c13]])
    m = np.array([0.0, mix.dm12sq, mix.dm12sq + mix.dm23sq])
    E = np.atleast_1d(E)
    ph = np.exp(-1j * 2.534 * m[None, :] * L_km / E[:, None])  # [ne, k]
    A = np.einsum("bk,nk,ak->nab", U, ph, U.conj())  # A[n, a, b] = amp(a->b)
    return (np.abs(A) ** 2).reshape(len(E), 9)  # channel a*3+b

"""Generate the golden fixtures in this folder from the reference itself.

Run in a container that holds the reference sources:

    make -C oracle ref            # compiles the reference's CPU propagators
    python tests/golden/make_golden.py

Every fixture is the output of the reference's AtmosCpuPropagator<double> /
BeamCpuPropagator<double> (through oracle/ref_shim.cpp), saved together with its inputs.
Layout: atmos ``out[type][ic][ie][9]``, beam ``out[type][ie][9]``; channel a*3+b = P(a->b);
type 0 = neutrino (knutype +1), 1 = antineutrino (knutype -1, NeutrinoType Antineutrino).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Mixing as OMix, Reference  # noqa: E402
from cudaprob3_gb300 import earth  # noqa: E402


def omix(m, knutype):
    return OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knutype)


def mix_array(m):
    return np.array([m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq])


def atmos_case(ref, name, mix, cz, en, model, h_km=22.0, poly=False, avg=None):
    if poly:
        radii, a, b, c, ye = model
        rho = np.zeros_like(radii)
        abc = (a, b, c)
    else:
        radii, rho, ye = model
        abc = None
        a = b = c = np.zeros_like(radii)
    outs = []
    for t, knu in ((0, 1), (1, -1)):
        av = None
        if avg is not None:
            av = (avg[0], avg[1], avg[2])
        outs.append(ref.atmos(omix(mix, knu), t == 1, cz, en, radii, rho, ye, h_km,
                              poly_abc=abc, avg=av, nthreads=4))
    extra = {}
    if avg is not None:
        extra = dict(avg_bins=np.int64(avg[0]), avg_prob=avg[1], avg_edges=avg[2])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), kind="atmos", mix=mix_array(mix),
                        cosines=cz, energies=en, radii=radii, rho=rho, a=a, b=b, c=c, ye=ye,
                        poly=np.int64(poly), h_km=np.float64(h_km), out=np.stack(outs), **extra)
    print(name, np.stack(outs).shape)


def beam_case(ref, name, mix, en, rho, L):
    outs = [ref.beam(omix(mix, knu), t == 1, en, rho, L, nthreads=4)
            for t, knu in ((0, 1), (1, -1))]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), kind="beam", mix=mix_array(mix),
                        energies=en, rho=np.float64(rho), L=np.float64(L), out=np.stack(outs))
    print(name, np.stack(outs).shape)


def main():
    if not Reference.available():
        sys.exit("build the reference first: make -C oracle ref")
    ref = Reference()
    nom = earth.NOMINAL
    io = earth.Mixing(nom.theta12, nom.theta13, nom.theta23, 0.7, nom.dm12sq, -2.49e-3)

    # headline atmospheric configuration on a reduced grid, and a subsample of the full grid
    atmos_case(ref, "atmos_prem4", nom, earth.cosine_grid(41), earth.log_energy_grid(33),
               earth.PREM_4LAYER)
    cz, en = earth.cosine_grid(400), earth.log_energy_grid(400)
    idx_c, idx_e = np.arange(0, 400, 19), np.arange(0, 400, 19)
    atmos_case(ref, "atmos_prem4_c0grid", nom, cz[idx_c], en[idx_e], earth.PREM_4LAYER)
    atmos_case(ref, "atmos_prem4_io", io, earth.cosine_grid(21), earth.log_energy_grid(17),
               earth.PREM_4LAYER)
    atmos_case(ref, "atmos_prem12", nom, earth.cosine_grid(25), earth.log_energy_grid(17),
               earth.PREM_12LAYER)
    atmos_case(ref, "atmos_shells59", nom, earth.cosine_grid(25), earth.log_energy_grid(17),
               earth.synthetic_shells(59))
    atmos_case(ref, "atmos_poly", nom, earth.cosine_grid(25), earth.log_energy_grid(17),
               earth.PREM_4LAYER_QUAD_V2, poly=True)
    # vacuum: every shell at zero density
    r, _, y = earth.PREM_4LAYER
    atmos_case(ref, "atmos_vacuum", nom, earth.cosine_grid(9), earth.log_energy_grid(9),
               (r, np.zeros_like(r), y))
    # mass degeneracy breaks (propagator.hpp:195-198)
    deg12 = earth.Mixing(nom.theta12, nom.theta13, nom.theta23, nom.dcp, 0.0, nom.dm23sq)
    deg23 = earth.Mixing(nom.theta12, nom.theta13, nom.theta23, nom.dcp, nom.dm12sq, 0.0)
    atmos_case(ref, "atmos_deg12", deg12, earth.cosine_grid(9), earth.log_energy_grid(9),
               earth.PREM_4LAYER)
    atmos_case(ref, "atmos_deg23", deg23, earth.cosine_grid(9), earth.log_energy_grid(9),
               earth.PREM_4LAYER)
    # edge cosines: shell-grazing limits, 0, tiny negatives, +-1; two production heights
    rr = earth.PREM_4LAYER[0][::-1]
    lim = -np.sqrt(1 - rr[1:] ** 2 / 6371.0 ** 2)
    edge = np.concatenate([[-1.0, -0.999999, 0.0, -1e-12, 1e-12, 1.0, 0.5],
                           lim, np.nextafter(lim, -2), np.nextafter(lim, 2)])
    atmos_case(ref, "atmos_edges", nom, edge, earth.log_energy_grid(7), earth.PREM_4LAYER)
    atmos_case(ref, "atmos_edges_h0", nom, edge, earth.log_energy_grid(5), earth.PREM_4LAYER,
               h_km=0.0)
    atmos_case(ref, "atmos_edges_h100", nom, edge, earth.log_energy_grid(5), earth.PREM_4LAYER,
               h_km=100.0)
    # production-height averaging (physics.hpp:997-1067, driven directly)
    rng = np.random.default_rng(7)
    ncz, nen, nb = 9, 7, 3
    w = rng.uniform(0.5, 1.5, (2, 3, nen, ncz, nb))
    w /= w.sum(axis=-1, keepdims=True)
    atmos_case(ref, "atmos_avg", nom, earth.cosine_grid(ncz), earth.log_energy_grid(nen),
               earth.PREM_4LAYER, avg=(nb, w.ravel(), np.array([10.0, 18.0, 25.0, 40.0])))

    # beam: headline baselines, the DUNE example of the reference, inverted ordering
    beam_case(ref, "beam_1300", nom, earth.lin_energy_grid(1001), 2.6, 1300.0)
    beam_case(ref, "beam_295", nom, earth.lin_energy_grid(1001), 2.6, 295.0)
    beam_case(ref, "beam_dune", nom, np.linspace(0.1, 500.0, 501), 2.848, 1284.9)
    beam_case(ref, "beam_io", io, earth.lin_energy_grid(501), 2.6, 1300.0)
    beam_case(ref, "beam_vacuum", nom, earth.lin_energy_grid(101), 0.0, 810.0)


if __name__ == "__main__":
    main()

"""Helpers for the GPU tests: run a golden fixture's inputs through the CUDA path."""
import numpy as np

from cudaprob3_gb300 import AtmosCudaPropagatorSingle, BeamCudaPropagatorSingle


def run_atmos(prec, mix6, knutype, anti, cz, en, radii, rho, ye, h_km, poly_abc=None):
    p = AtmosCudaPropagatorSingle(0, len(cz), len(en), precision=prec)
    p.setEnergyList(en)
    p.setCosineList(cz)
    p.setMNSMatrix(mix6[0], mix6[1], mix6[2], mix6[3], knutype)
    p.setNeutrinoMasses(mix6[4], mix6[5])
    if poly_abc is not None:
        p.setDensity(radii, poly_abc[0], poly_abc[1], poly_abc[2], ye)
    else:
        p.setDensity(radii, rho, ye)
    p.setProductionHeight(h_km)
    p.calculateProbabilities(1 if anti else 0)
    return p.probabilities()


def run_beam(prec, mix6, knutype, anti, en, rho, L):
    b = BeamCudaPropagatorSingle(0, len(en), 1, precision=prec)
    b.setEnergyList(en)
    b.setMNSMatrix(mix6[0], mix6[1], mix6[2], mix6[3], knutype)
    b.setNeutrinoMasses(mix6[4], mix6[5])
    b.setDensity(rho)
    b.setPathLength(L)
    b.calculateProbabilities(1 if anti else 0)
    return b.probabilities()


def run_fixture(d, prec):
    outs = []
    for t, knu in ((0, 1), (1, -1)):
        if str(d["kind"]) == "atmos":
            abc = (d["a"], d["b"], d["c"]) if int(d["poly"]) else None
            outs.append(run_atmos(prec, d["mix"], knu, t == 1, d["cosines"], d["energies"],
                                  d["radii"], d["rho"], d["ye"], float(d["h_km"]), abc))
        else:
            outs.append(run_beam(prec, d["mix"], knu, t == 1, d["energies"], float(d["rho"]),
                                 float(d["L"])))
    return np.stack(outs)

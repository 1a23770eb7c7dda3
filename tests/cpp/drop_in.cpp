// Drop-in check of the C++ facade: the reference's example call order
// (example/mainatmos.cpp:111-160, example/mainbeam.cpp:107-142) against
// include/cudaprob3_gb300.hpp.  Prints "atmos ic ie t value" / "beam ie t value" lines that
// the GPU test compares with the oracle.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cudaprob3_gb300.hpp"

using namespace cudaprob3linear;

int main(int argc, char** argv) {
    const char* model = argc > 1 ? argv[1] : nullptr;
    const int nc = 20, ne = 16;
    std::vector<double> cz(nc), en(ne);
    for (int i = 0; i < nc; i++) cz[i] = -1.0 + 2.0 * i / (nc - 1);
    for (int i = 0; i < ne; i++) en[i] = std::pow(10.0, -1.0 + 3.0 * i / (ne - 1));

    AtmosCudaPropagatorSingle* propagator = new AtmosCudaPropagatorSingle(0, nc, ne);
    propagator->setEnergyList(en);
    propagator->setCosineList(cz);
    propagator->setMNSMatrix(0.5843, 0.1496, 0.7365, -1.601, 1);
    propagator->setNeutrinoMasses(7.53e-5, 2.49e-3);
    if (model)
        propagator->setDensityFromFile(model);
    else
        propagator->setDensity({0., 1220., 3480., 5701., 6371.}, {13., 13., 11.3, 5., 3.3},
                               {.468, .468, .468, .497, .497});
    propagator->setProductionHeight(22.0);
    std::printf("boundaries %d\n", propagator->getNlayerBoundaries());
    propagator->calculateProbabilities(cudaprob3linear::Neutrino);
    for (int ic = 0; ic < nc; ic += 3)
        for (int ie = 0; ie < ne; ie += 5)
            for (int t = 0; t < 9; t++)
                std::printf("atmos %d %d %d %.17g\n", ic, ie, t,
                            propagator->getProbability(ic, ie, ProbType(t)));
    try {
        propagator->getProbability(nc, 0, ProbType::e_e);
        std::printf("no exception\n");
        return 1;
    } catch (const std::runtime_error& e) {
        std::printf("caught: %s\n", e.what());
    }
    delete propagator;

    CudaPropagatorSingle<float> mixed(0, nc, ne);  // legacy template name, float -> mixed
    (void)mixed;

    BeamCudaPropagatorSingle beam(0, 1000, 1);
    std::vector<double> eb(1000);
    for (int i = 0; i < 1000; i++) eb[i] = 0.1 + 9.9 * i / 999.0;
    beam.setEnergyList(eb);
    beam.setMNSMatrix(0.5843, 0.1496, 0.7365, -1.601, 1);
    beam.setNeutrinoMasses(7.53e-5, 2.49e-3);
    beam.setDensity(2.6);
    beam.setPathLength(1300.0);
    beam.calculateProbabilities(cudaprob3linear::Neutrino);
    for (int ie = 0; ie < 1000; ie += 111)
        for (int t = 0; t < 9; t++) std::printf("beam %d %d %.17g\n", ie, t, beam.getProbability(ie, ProbType(t)));
    return 0;
}

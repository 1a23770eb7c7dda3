// Includes the reference's header names and uses its classes and constants.
#include <atmoscudapropagator.cuh>
#include <beamcudapropagator.cuh>

#include <cstdio>

using namespace cudaprob3linear;

int main() {
    std::printf("REarth %g, max shells %d\n", Constants<double>::REarth(), Constants<double>::MaxNLayers());
    try {
        AtmosCudaPropagatorSingle p(0, 4, 4);
        BeamCudaPropagatorSingle b(0, 4, 1);
        (void)p;
        (void)b;
        std::printf("created\n");
    } catch (const std::runtime_error& e) {
        std::printf("runtime_error: %s\n", e.what());
    }
    return 0;
}

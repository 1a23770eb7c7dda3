// The C++ wrappers of batches and the serving loop: one batch of two atmospheric problems
// and one beam problem, then three served requests; prints values for the test to check.
#include <cmath>
#include <cstdio>
#include <vector>

#include "cudaprob3_gb300.hpp"

using namespace cudaprob3linear;

static std::vector<double> lin(double a, double b, int n) {
    std::vector<double> v(n);
    for (int i = 0; i < n; i++) v[i] = a + (b - a) * i / (n - 1);
    return v;
}
static std::vector<double> logs(double a, double b, int n) {
    std::vector<double> v(n);
    for (int i = 0; i < n; i++) v[i] = std::pow(10.0, std::log10(a) + (std::log10(b) - std::log10(a)) * i / (n - 1));
    return v;
}

int main() {
    const std::vector<double> radii{0.0, 1220.0, 3480.0, 5701.0, 6371.0};
    const std::vector<double> rho{13.0, 13.0, 11.3, 5.0, 3.3};
    const std::vector<double> ye{0.468, 0.468, 0.468, 0.497, 0.497};
    const double t12 = 0.5843, t13 = 0.1496, t23 = 0.7365, dcp = -1.601, dm12 = 7.53e-5,
                 dm23 = 2.49e-3;
    const std::vector<double> cz = lin(-1.0, 1.0, 20), en = logs(0.1, 100.0, 16);
    const std::vector<double> eb = lin(0.1, 10.0, 1000);

    PropagatorBatch b(0);
    b.setEarth(radii, rho, ye, 22.0);
    const int a0 = b.addAtmospheric(cz, en), a1 = b.addAtmospheric(cz, en);
    const int bm = b.addBeam(eb, 2.6, {1300.0});
    b.setParameters(a0, t12, t13, t23, dcp, 1, dm12, dm23, Neutrino);
    b.setParameters(a1, t12, t13, t23, dcp, -1, dm12, dm23, Antineutrino);
    b.setParameters(bm, t12, t13, t23, dcp, 1, dm12, dm23, Neutrino);
    b.commit();
    b.run();
    b.synchronize();
    const std::vector<float> r0 = b.result(a0), r1 = b.result(a1), rb = b.result(bm);
    // atmospheric layout [9][nc][ne]; beam [n_baselines][9][ne]
    for (int t = 0; t < 9; t++)
        for (int ic = 0; ic < 20; ic += 3)
            for (int ie = 0; ie < 16; ie += 5) {
                std::printf("batch_nu %d %d %d %.9g\n", ic, ie, t, r0[(t * 20 + ic) * 16 + ie]);
                std::printf("batch_nubar %d %d %d %.9g\n", ic, ie, t, r1[(t * 20 + ic) * 16 + ie]);
            }
    for (int t = 0; t < 9; t++)
        for (int ie = 0; ie < 1000; ie += 97) std::printf("batch_beam %d %d %.9g\n", ie, t, rb[t * 1000 + ie]);

    PropagatorServer s(0, (size_t)256 << 20);
    s.setEarth(radii, rho, ye, 22.0);
    const int g = s.addAtmosphericGrid(cz, en);
    s.start();
    std::vector<unsigned long long> ids;
    s.poll(0, 0.0);  // start recording completions
    for (int k = 0; k < 3; k++) ids.push_back(s.submit(g, t12, t13, t23, dcp, 1, dm12, dm23, Neutrino));
    std::vector<unsigned long long> finished;
    for (int tries = 0; finished.size() < ids.size() && tries < 600; tries++)
        for (unsigned long long id : s.poll(8, 0.05)) finished.push_back(id);
    if (finished.size() != ids.size()) {
        std::printf("timeout\n");
        return 1;
    }
    for (unsigned long long id : ids) {
        if (!s.wait(id, 0.0)) {
            std::printf("timeout\n");
            return 1;
        }
        double lat = 0.0;
        const std::vector<float> r = s.result(id, &lat);
        for (int t = 0; t < 9; t++)
            for (int ic = 0; ic < 20; ic += 3)
                for (int ie = 0; ie < 16; ie += 5)
                    std::printf("served %d %d %d %.9g\n", ic, ie, t, r[(t * 20 + ic) * 16 + ie]);
        s.release(id);
    }
    try {
        b.result(7);
    } catch (const std::runtime_error& e) {
        std::printf("caught: %s\n", e.what());
    }
    return 0;
}

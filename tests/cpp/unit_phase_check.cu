// Host checks of the mixed kernels' phase arithmetic in turns (cp3_device.cuh, callable from
// the host).
//  1. unit_turn_minus_one: z = e^{-2 pi i (r + lo)} - 1 over |r| up to 1/2 turn plus the
//     overshoot the final Fast2Sum can leave, with remainders lo of either sign, including
//     ulp steps around the branch points, against double precision: error <= 3e-7.
//  2. reduced_turn: the reduced product of double-float phase rates and lengths over the
//     ranges of the kernels (up to ~200 turns), against the product reduced in long double
//     arithmetic: error <= 1e-10 turns.
// Prints the largest errors; exit status 1 above either bound.
#include <cmath>
#include <cstdio>
#include <random>

#include "cp3_device.cuh"

int main() {
    const double two_pi = 6.283185307179586476925286766559;
    double worst = 0.0, at = 0.0;
    auto check = [&](float r, float lo) {
        float zre, zim;
        cp3::unit_turn_minus_one(r, lo, zre, zim);
        const double ph = two_pi * ((double)r + (double)lo);
        const double er = std::fabs((double)zre - (std::cos(ph) - 1.0));
        const double ei = std::fabs((double)zim + std::sin(ph));
        const double e = er > ei ? er : ei;
        if (e > worst) {
            worst = e;
            at = r;
        }
    };
    for (int i = -400000; i <= 400000; i++) {  // a dense sweep of [-1/2 - 2e-4, 1/2 + 2e-4]
        const float r = (float)((0.5 + 2e-4) * i / 400000.0);
        check(r, 0.0f);
        check(r, 2e-8f);
        check(r, -2e-8f);
    }
    for (float r0 : {0.5f, -0.5f, 0.25f, -0.25f, 0.0f}) {
        float r = r0;  // ulp steps either side of the branch points
        for (int k = 0; k < 2000; k++) {
            check(r, 0.0f);
            r = std::nextafter(r, 10.0f);
        }
        r = r0;
        for (int k = 0; k < 2000; k++) {
            check(r, 0.0f);
            r = std::nextafter(r, -10.0f);
        }
    }
    std::printf("unit_turn_minus_one: max |z - exact| = %.3e at r = %.9g\n", worst, at);

    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> rate(1e-4, 0.05), len(1.0, 13000.0);
    double worst_t = 0.0;
    for (int i = 0; i < 2000000; i++) {
        const double w = rate(rng), L = len(rng);
        const float wh = (float)w, wl = (float)(w - (double)wh);
        const float Lh = (float)L, Ll = (float)(L - (double)Lh);
        float lo;
        const float s = cp3::reduced_turn(wh, wl, Lh, Ll, lo);
        const long double t = ((long double)wh + wl) * ((long double)Lh + Ll);
        const long double red = t - std::nearbyint((double)t);
        long double d = (long double)s + lo - red;
        d -= std::nearbyint((double)d);  // same point of the circle
        const double e = std::fabs((double)d);
        if (e > worst_t) worst_t = e;
    }
    std::printf("reduced_turn: max error = %.3e turns\n", worst_t);
    return (worst <= 3e-7 && worst_t <= 1e-10) ? 0 : 1;
}

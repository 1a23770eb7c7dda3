// Host check of the mixed kernels' unit phase factor z = e^{-i (r + lo)} - 1
// (unit_phase_minus_one, cp3_device.cuh, callable from the host): over |r| up to pi plus
// the overshoot the FP32 range reduction can leave (arguments within rounding of a
// half-turn), with remainders lo of either sign, against double precision.  Prints the
// largest error; exit status 1 above 3e-7.
#include <cmath>
#include <cstdio>

#include "cp3_device.cuh"

int main() {
    double worst = 0.0, at = 0.0;
    const double pi = 3.14159265358979323846;
    auto check = [&](float r, float lo) {
        float zre, zim;
        cp3::unit_phase_minus_one(r, lo, zre, zim);
        const double ph = (double)r + (double)lo;
        const double er = std::fabs((double)zre - (std::cos(ph) - 1.0));
        const double ei = std::fabs((double)zim + std::sin(ph));
        const double e = er > ei ? er : ei;
        if (e > worst) {
            worst = e;
            at = r;
        }
    };
    for (int i = -400000; i <= 400000; i++) {  // a dense sweep of [-pi - 1e-3, pi + 1e-3]
        const float r = (float)((pi + 1e-3) * i / 400000.0);
        check(r, 0.0f);
        check(r, 1.1e-7f);
        check(r, -1.1e-7f);
    }
    for (float r0 : {(float)pi, (float)(-pi), 1.5707964f, -1.5707964f, 0.0f}) {
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
    std::printf("max |z - exact| = %.3e at r = %.9g\n", worst, at);
    return worst <= 3e-7 ? 0 : 1;
}

// cp3_f64.cuh -- building blocks of the FP64 kernels in the rotated real basis: one layer as
// S = 1 + z1 u1 u1^T + z2 u2 u2^T with the reference's own phases, the layer matrix, and the
// flavour-basis amplitude A = W A2 W^+.  Shared by the atmospheric kernels (cp3_atmos.cu) and
// the beam kernel (cp3_tables.cu, which is compiled without FMA contraction).
#pragma once

#include "cp3_device.cuh"

namespace cp3 {

struct cm3 {
    cd a[3][3];
};

// One FP64 layer in factored form.
struct Layer64 {
    double u[2][3];  // unit eigenvectors u1, u2 (rotated basis)
    cd z[2];         // e^{i (arg_k - arg_0)} - 1, k = 1, 2
};

// The phases of one layer from dmMatVac[k][0], as getArg (physics.hpp:439-450) evaluates
// them; arg[] receives arg_k.  The relative phase arg_k - arg_0 is taken exactly, as a
// TwoSum pair dh + dl (a rounded difference could be off by 1e-13 rad at ~800 rad, which
// ~120 layers would accumulate), and e^{i(dh + dl)} = e^{i dh} (1 + i dl) to second order in
// |dl| <= 1e-13: two sincos per layer instead of the three of multiply_phase_matrix
// (math.hpp:59-75), with the reference's relative phases to ~1e-16.
// x / E, correctly rounded, from rE = 1/E correctly rounded: q = x rE, then one correction
// with the exact residual x - q E (an FMA).  By Markstein's theorem (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34, 1990) the corrected quotient is the correctly rounded x / E; an exhaustive-style
// check against IEEE division (4e8 random and edge-significand operand pairs) found no
// difference.  Three FP64 instructions instead of a full division: the reference's phase
// roundings at a fraction of the cost on GB300's narrow FP64 pipe.
__device__ __forceinline__ double div_by(double x, double E, double rE) {
    const double q = __dmul_rn(x, rE);
    return fma(fma(-q, E, x), rE, q);
}

__device__ __forceinline__ void layer64_phases(const double dmv[3], double L, double E,
                                               double rE, Layer64& f, double arg[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) arg[k] = div_by(__dmul_rn(__dmul_rn(-kLoEFac, dmv[k]), L), E, rE);
#pragma unroll
    for (int kk = 0; kk < 2; kk++) {
        const int k = kk + 1;
        const double dh = __dadd_rn(arg[k], -arg[0]);  // TwoSum (Knuth)
        const double bb = __dadd_rn(dh, -arg[k]);
        const double dl = __dadd_rn(__dadd_rn(arg[k], -__dadd_rn(dh, -bb)), __dadd_rn(-arg[0], -bb));
        double s, c;
        sincos(dh, &s, &c);
        // e^{i dh} (1 + i dl) - 1
        f.z[kk] = cd{(c - 1.0) - s * dl, s + c * dl};
    }
}

// G = S
__device__ __forceinline__ void layer_to_gen64(const Layer64& f, cm3& G) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const double p0 = f.u[0][i] * f.u[0][j], p1 = f.u[1][i] * f.u[1][j];
            const cd v{(i == j ? 1.0 : 0.0) + f.z[0].re * p0 + f.z[1].re * p1,
                       f.z[0].im * p0 + f.z[1].im * p1};
            G.a[i][j] = v;
            G.a[j][i] = v;
        }
}

// Flavour-basis amplitude A = W A2 W^+, W = [[1,0,0],[0,c,s e],[0,-s,c e]], e = e^{i d}.
__device__ __forceinline__ void to_flavour64(const cm3& A2, const double* w, cm3& A) {
    const double c = w[0], s = w[1], er = w[2], ei = w[3];
    cm3 Y;  // A2 W^+
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const cd a1 = A2.a[i][1], a2 = A2.a[i][2];
        const cd f{a2.re * er + a2.im * ei, a2.im * er - a2.re * ei};  // e* a2
        Y.a[i][0] = A2.a[i][0];
        Y.a[i][1] = cd{c * a1.re + s * f.re, c * a1.im + s * f.im};
        Y.a[i][2] = cd{-s * a1.re + c * f.re, -s * a1.im + c * f.im};
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const cd y1 = Y.a[1][j], y2 = Y.a[2][j];
        const cd g{y2.re * er - y2.im * ei, y2.re * ei + y2.im * er};  // e y2
        A.a[0][j] = Y.a[0][j];
        A.a[1][j] = cd{c * y1.re + s * g.re, c * y1.im + s * g.im};
        A.a[2][j] = cd{-s * y1.re + c * g.re, -s * y1.im + c * g.im};
    }
}

}  // namespace cp3

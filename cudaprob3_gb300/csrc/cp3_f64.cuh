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

// The nine probabilities of a single constant-density layer (a beam baseline, or an
// atmospheric bin that crosses no shell) from the three-flavour expansion over the matter
// eigenstates, in FP64: the form of layer_coefficients / layer_store in cp3_mixed.cuh.
//   P(a -> b) = delta_ab + 2 sum_{j>k} [Re c_jk (cos D_jk - 1) + Im c_jk sin D_jk],
// with c_jk = m_aj m_ak for a = b (m_ak = |U_ak|^2, U_ak = (W u_k)_a); for a != b,
// Re c_jk = W_l - (W_0 + W_1 + W_2) / 2 (W_k = m_ak m_bk, l the third index) and
// Im c_10 = -Im c_20 = Im c_21 = +-J, the matter Jarlskog invariant (+ for e->mu, mu->tau,
// tau->e).  It replaces forming S and its flavour-basis product (about 150 FP64 operations
// per path length) by 19 coefficients per (energy, density) and about 30 operations per
// path length.
struct LayerCoefs64 {
    double d[3][3];  // flavour a's survival: 2 m_aj m_ak for (j, k) = (1, 0), (2, 0), (2, 1)
    double o[3][3];  // the pairs (e, mu), (mu, tau), (tau, e): 2 Re c_jk for the same (j, k)
    double j2;       // 2 J_{e mu}
};

// u[k-1]: the unit eigenvector of eigenstate k in the rotated basis; w = {c23, s23, cos d, sin d}.
__device__ __forceinline__ LayerCoefs64 layer_coefficients64(const double u[2][3], const double* w) {
    const double c = w[0], s = w[1], er = w[2], ei = w[3];
    const double cc = c * c, ss = s * s, cs2 = 2.0 * c * s;
    double m[3][2], m0[3];  // m[a][k-1] = |U_ak|^2, m0[a] = |U_a0|^2
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const double b1 = u[k][1] * u[k][1], b2 = u[k][2] * u[k][2], xr = u[k][1] * u[k][2] * (cs2 * er);
        m[0][k] = u[k][0] * u[k][0];
        m[1][k] = cc * b1 + ss * b2 + xr;
        m[2][k] = ss * b1 + cc * b2 - xr;
    }
#pragma unroll
    for (int a = 0; a < 3; a++) m0[a] = 1.0 - m[a][0] - m[a][1];
    LayerCoefs64 q;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        q.d[a][0] = 2.0 * m0[a] * m[a][0];
        q.d[a][1] = 2.0 * m0[a] * m[a][1];
        q.d[a][2] = 2.0 * m[a][0] * m[a][1];
    }
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const int a = p, b = p == 2 ? 0 : p + 1;
        const double W0 = m0[a] * m0[b], W1 = m[a][0] * m[b][0], W2 = m[a][1] * m[b][1];
        const double S = W0 + W1 + W2;
        q.o[p][0] = 2.0 * W2 - S;
        q.o[p][1] = 2.0 * W1 - S;
        q.o[p][2] = 2.0 * W0 - S;
    }
    q.j2 = cs2 * ei * (u[0][0] * u[1][0]) * (u[0][1] * u[1][2] - u[0][2] * u[1][1]);
    return q;
}

// The nine probabilities of one path length from the coefficients and the layer's
// z_k = e^{-i phi_k} - 1; channel a*3+b = P(a -> b) at out[ch * plane].
__device__ __forceinline__ void layer_store64(const LayerCoefs64& q, const cd z[2],
                                              double* __restrict__ out, size_t plane) {
    // cos D - 1 for (1,0), (2,0), (2,1); sin D_10 - sin D_20 + sin D_21 = Im z_1 Re z_2 - Im z_2 Re z_1
    const double g0 = z[0].re, g1 = z[1].re;
    const double g2 = z[0].re + z[1].re + z[0].re * z[1].re + z[0].im * z[1].im;
    const double jt = q.j2 * (z[0].im * z[1].re - z[1].im * z[0].re);
#pragma unroll
    for (int a = 0; a < 3; a++)
        out[(size_t)(a * 4) * plane] = 1.0 + q.d[a][0] * g0 + q.d[a][1] * g1 + q.d[a][2] * g2;
    // (e, mu): channels 1 (e->mu) and 3 (mu->e); (mu, tau): 5 and 7; (tau, e): 6 and 2
    constexpr int fwd[3] = {1, 5, 6}, rev[3] = {3, 7, 2};
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const double v = q.o[p][0] * g0 + q.o[p][1] * g1 + q.o[p][2] * g2;
        out[(size_t)fwd[p] * plane] = v + jt;
        out[(size_t)rev[p] * plane] = v - jt;
    }
}

}  // namespace cp3

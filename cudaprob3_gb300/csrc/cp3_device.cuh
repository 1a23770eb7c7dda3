// cp3_device.cuh -- device building blocks shared by the kernels.
//
// Part 1 (FP64, reference-faithful): the matter eigenvalues, spectral products and
// flavour-basis projectors of physics.hpp, in the reference's evaluation order.  Used by
// the FP64 tables/kernels and by the FP64 eigen-decomposition of the mixed tables.
// Part 2 (mixed): double-float phase products and range reduction, complex float helpers.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "cp3_types.h"

namespace cp3 {

// Pure arithmetic: callable from the host as well (the CPU checks of the mixed solver).
#define CP3_HD __host__ __device__ __forceinline__

// Separately rounded float product / sum, never fused by the compiler: the error-free
// transformations below rely on it (a product contracted into the following addition
// would make TwoSum / Fast2Sum / TwoProduct inexact).
#ifdef __CUDA_ARCH__
#define CP3_FMUL(a, b) __fmul_rn((a), (b))
#define CP3_FADD(a, b) __fadd_rn((a), (b))
#else
#define CP3_FMUL(a, b) ((a) * (b))
#define CP3_FADD(a, b) ((a) + (b))
#endif

struct cd {
    double re, im;
};
struct cf {
    float re, im;
};

#define CP3_U(p, i, j) (cd{(p)->U[((i)*3 + (j)) * 2], (p)->U[((i)*3 + (j)) * 2 + 1]})
#define CP3_DM(p, i, j) ((p)->dm[(i)*3 + (j)])

// physics::getMfast (physics.hpp:267-340): matter eigenvalues of 2E.H (eV^2), ordered by the
// vacuum root order.  Returns mm[i]; the reference's dmMatVac[i][j] = mm[i] - DM(j,0) and
// dmMatMat[i][j] = mm[i] - mm[j].
CP3_HD void matter_masses_f64(const OscParams* __restrict__ p, double E,
                                                  double rho, double mm[3]) {
    const double fac = p->anti ? kTwoRtTwoGf * E * rho : -kTwoRtTwoGf * E * rho;
    const double d01 = CP3_DM(p, 0, 1), d02 = CP3_DM(p, 0, 2);
    const cd u00 = CP3_U(p, 0, 0), u01 = CP3_U(p, 0, 1), u02 = CP3_U(p, 0, 2);
    const double alpha = fac + d01 + d02;
    const double beta = d01 * d02 + fac * (d01 * (1.0 - u01.re * u01.re - u01.im * u01.im) +
                                           d02 * (1.0 - u02.re * u02.re - u02.im * u02.im));
    const double gamma = fac * d01 * d02 * (u00.re * u00.re + u00.im * u00.im);
    const double tmp = alpha * alpha - 3.0 * beta < 0 ? 0 : alpha * alpha - 3.0 * beta;
    const double argtmp = (2.0 * alpha * alpha * alpha - 9.0 * alpha * beta + 27.0 * gamma) /
                          (2.0 * sqrt(tmp * tmp * tmp));
    const double arg = fabs(argtmp) > 1.0 ? argtmp / fabs(argtmp) : argtmp;
    const double th0 = acos(arg) / 3.0;
    const double th1 = th0 - (2.0 * M_PI / 3.0);
    const double th2 = th0 + (2.0 * M_PI / 3.0);
    double r[3];
    r[0] = -(2.0 / 3.0) * sqrt(tmp);
    r[1] = -(2.0 / 3.0) * sqrt(tmp);
    r[2] = -(2.0 / 3.0) * sqrt(tmp);
    r[0] *= cos(th0);
    r[1] *= cos(th1);
    r[2] *= cos(th2);
    const double shift = CP3_DM(p, 0, 0) - alpha / 3.0;
    r[0] += shift;
    r[1] += shift;
    r[2] += shift;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int o = p->order[i];
        mm[i] = o == 0 ? r[0] : (o == 1 ? r[1] : r[2]);
    }
}

// Index of (i, j), i <= j, in the 6-entry storage of a symmetric 3x3 matrix.
__host__ __device__ constexpr int sidx(int i, int j) {
    return i <= j ? (i == 0 ? j : (i == 1 ? 2 + j : 5)) : (j == 0 ? i : (j == 1 ? 2 + i : 5));
}

// Eigen-decomposition used by the mixed kernels, in FP64.  In the basis rotated by
// W = R23 . diag(1,1,e^{i d}) the Hamiltonian 2E.H is the real symmetric H0 + V e0 e0^T
// (V = -fac of getMfast).  Eigenvalues come from the reference cubic (matter_masses_f64,
// same spectrum); the projectors onto the eigenvalues k = 1, 2 are
//   P_k = (H - m_a)(H - m_b) / ((m_k - m_a)(m_k - m_b)),  {a, b} = the other two,
// (P_0 = 1 - P_1 - P_2), and the phase rates relative to eigenvalue 0 are
//   omega_k = 2.534 (m_k - m_0) / E   [rad / km]
// (the mixed kernels' fallback hands them on in turns per km, omega_k / (2 pi)).
// Projectors P1, P2 (00,01,02,11,12,22) of the rotated H for the matter masses mm (in the
// reference's mass order).
CP3_HD void rotated_projectors_f64(const OscParams* __restrict__ p, double E, double rho,
                                   const double mm[3], double P[2][6]) {
    const double fac = p->anti ? kTwoRtTwoGf * E * rho : -kTwoRtTwoGf * E * rho;
    double h[6];
#pragma unroll
    for (int q = 0; q < 6; q++) h[q] = p->h0[q];
    h[0] -= fac;
#pragma unroll
    for (int kk = 0; kk < 2; kk++) {
        const int k = kk + 1;
        const int a = 0;
        const int b = k == 1 ? 2 : 1;
        double A[6], B[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
            A[q] = h[q];
            B[q] = h[q];
        }
        A[0] -= mm[a];
        A[3] -= mm[a];
        A[5] -= mm[a];
        B[0] -= mm[b];
        B[3] -= mm[b];
        B[5] -= mm[b];
        const double inv = 1.0 / ((mm[k] - mm[a]) * (mm[k] - mm[b]));
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) {
                double s = 0.0;
#pragma unroll
                for (int m = 0; m < 3; m++) s += A[sidx(i, m)] * B[sidx(m, j)];
                P[kk][sidx(i, j)] = s * inv;
            }
    }
}

CP3_HD void rotated_eigen_f64(const OscParams* __restrict__ p, double E,
                                                  double rho, double P[2][6], double om[2]) {
    double mm[3];
    matter_masses_f64(p, E, rho, mm);
    rotated_projectors_f64(p, E, rho, mm, P);
#pragma unroll
    for (int kk = 0; kk < 2; kk++) om[kk] = kLoEFac * (mm[kk + 1] - mm[0]) / E;
}

// Unit vector u with P = u u^T from a rank-one projector P (sign arbitrary): the column j of
// P with the largest diagonal, over sqrt(P[j][j]).
template <class T>
CP3_HD void projector_vector(const T P[6], T u[3]) {
    const T d0 = P[0], d1 = P[3], d2 = P[5];
    const int j = (d0 >= d1 && d0 >= d2) ? 0 : (d1 >= d2 ? 1 : 2);
    const T c0 = j == 0 ? d0 : (j == 1 ? P[1] : P[2]);
    const T c1 = j == 0 ? P[1] : (j == 1 ? d1 : P[4]);
    const T c2 = j == 0 ? P[2] : (j == 1 ? P[4] : d2);
    const T rs = (T)1 / sqrt(j == 0 ? d0 : (j == 1 ? d1 : d2));
    u[0] = c0 * rs;
    u[1] = c1 * rs;
    u[2] = c2 * rs;
}

// ---------------------------------------------------------------------------------------
// Mixed-precision helpers.

// Phases in turns.  The mixed kernels carry every phase rate as omega / (2 pi) (turns per
// km), so that a phase t = omega L is reduced by subtracting an integer: with t = p + e the
// double-float product (p its float part), n = rint(p) and p - n are exact, and the reduced
// phase (p - n) + e keeps the product's full accuracy (~1e-11 turns for |t| < 1e3).  A
// reduction in radians, by a float 2 pi split in parts, rounds its remainder once more
// (~1e-8 turns), and over the ~120 layers of a core-crossing trajectory that rounding was
// the largest error term.

// Double-float product t = (ah + al)(bh + bl) reduced to [-1/2, 1/2] turns, returned as
// r + lo with |lo| <= ulp(r)/2.  The exact product of the leading parts comes from an FMA
// (Dekker/Ogita TwoProduct), the cross terms go to the error word, the integer part is
// subtracted exactly, and the last addition's remainder is kept.
CP3_HD float reduced_turn(float ah, float al, float bh, float bl, float& lo) {
    const float p = CP3_FMUL(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    const float f = CP3_FADD(p, -rintf(p));  // exact
    const float s = CP3_FADD(f, e);
    lo = CP3_FADD(CP3_FADD(f, -s), e);  // Fast2Sum remainder (second order where |f| < |e|)
    return s;
}

// sin(2 pi x) and cos(2 pi x) for 0 <= x <= 1/4 (turns):
//   s = x (S1 + x^2 P(x^2)),  c = 1 + x^2 (C2 + x^2 Q(x^2)),
// S1 = 2 pi and C2 = -2 pi^2 as float pairs (hi + lo: a float 2 pi alone would put a
// systematic 3e-8 into every angle), P and Q of degree 3, Horner form with FMA.  P and Q are
// near-minimax fits on [0, 1/4] made for this file (Lawson-reweighted least squares on
// Chebyshev nodes, fit_sincos.py beside it); with every coefficient rounded to float the
// angle of (s, c) is off by at most 4e-9 rad, under the FP32 rounding of the evaluation.
constexpr float kS1Hi = 6.283185482e+00f, kS1Lo = -1.748455531e-07f;
constexpr float kC2Hi = -1.973920822e+01f, kC2Lo = -5.807431762e-07f;
constexpr float kP3 = -4.134167862e+01f, kP5 = 8.160215759e+01f, kP7 = -7.657188416e+01f,
                kP9 = 3.968270874e+01f;
constexpr float kQ4 = 6.493937683e+01f, kQ6 = -8.545484924e+01f, kQ8 = 6.016622543e+01f,
                kQ10 = -2.511871529e+01f;
constexpr float kTwoPiF = 6.283185482e+00f;
constexpr float kPiF = 3.141592741e+00f;

CP3_HD void poly_sincos_turns(float x, float& s, float& c) {
    const float x2 = x * x;
    float ps = fmaf(kP9, x2, kP7);
    ps = fmaf(ps, x2, kP5);
    ps = fmaf(ps, x2, kP3);
    ps = fmaf(ps, x2, kS1Lo);  // S1lo + x^2 P
    s = fmaf(x, kS1Hi, x * ps);
    float pc = fmaf(kQ10, x2, kQ8);
    pc = fmaf(pc, x2, kQ6);
    pc = fmaf(pc, x2, kQ4);
    pc = fmaf(pc, x2, kC2Lo);  // C2lo + x^2 Q
    c = fmaf(x2, pc, fmaf(x2, kC2Hi, 1.0f));
}

// z = e^{-2 pi i (r + lo)} - 1 for |r| <= 1/2 turn (+ a little: the Fast2Sum can leave |r|
// just past 1/2).  |r| > 1/4 is reflected through 1/2 (1/2 - |r| is exact by Sterbenz);
// past 1/2 the reflected argument is negative and so is its sine, which is why the sign of r
// multiplies sin instead of replacing its sign.  The remainder lo enters to first order:
// e^{-2 pi i lo} = 1 - 2 pi i lo.  (s, c) are not renormalised: the fitted polynomials give
// s^2 + c^2 = 1 to the FP32 rounding already, and a renormalisation through rsqrt measured
// slower and, with its own roundings, less accurate (59-shell grid max error 3.15e-6 with
// it, 2.6e-6 without).
CP3_HD void unit_turn_minus_one(float r, float lo, float& zre, float& zim) {
    const float a = fabsf(r);
    const bool refl = a > 0.25f;
    const float x = refl ? 0.5f - a : a;
    float sx, cx;
    poly_sincos_turns(x, sx, cx);
    const float sn = r < 0.0f ? -sx : sx;
    const float cs = refl ? -cx : cx;
    const float ml = -kTwoPiF * lo;
    zre = fmaf(ml, sn, cs - 1.0f);
    zim = fmaf(ml, cs, -sn);
}

// ---------------------------------------------------------------------------------------
// Double-float ("df64") arithmetic on the FP32 pipe: a value is hi + lo with |lo| <=
// ulp(hi)/2, ~48 significant bits.  Error-free transformations: TwoSum (Knuth),
// Fast2Sum (Dekker), TwoProduct through FMA; the sums are the "sloppy" variant (one
// renormalisation), which is accurate to a few df64 ulps of the larger operand.

struct df {
    float hi, lo;
};

CP3_HD df df_from(double x) {
    const float h = (float)x;
    return df{h, (float)(x - (double)h)};
}
#ifdef __CUDACC__
CP3_HD df to_df(double x) { return df_from(x); }
CP3_HD df to_df(float2 x) { return df{x.x, x.y}; }  // already split on the host
#endif
CP3_HD df df_fast2sum(float a, float b) {  // |a| >= |b|
    const float s = CP3_FADD(a, b);
    return df{s, CP3_FADD(b, -CP3_FADD(s, -a))};
}
CP3_HD df df_add(df x, df y) {
    const float s = CP3_FADD(x.hi, y.hi);
    const float bb = CP3_FADD(s, -x.hi);
    float e = CP3_FADD(CP3_FADD(x.hi, -CP3_FADD(s, -bb)), CP3_FADD(y.hi, -bb));
    e = CP3_FADD(e, CP3_FADD(x.lo, y.lo));
    return df_fast2sum(s, e);
}
CP3_HD df df_neg(df x) { return df{-x.hi, -x.lo}; }
CP3_HD df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
CP3_HD df df_mul(df x, df y) {
    const float p = CP3_FMUL(x.hi, y.hi);
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return df_fast2sum(p, e);
}
CP3_HD df df_mulf(df x, float y) {
    const float p = CP3_FMUL(x.hi, y);
    const float e = fmaf(x.hi, y, -p);
    return df_fast2sum(p, fmaf(x.lo, y, e));
}
// 1 / x to df64 accuracy: float reciprocal, then one Newton step in df64.
CP3_HD df df_recip(df x) {
    const float r = 1.0f / x.hi;
    const df one_minus = df_sub(df{1.0f, 0.0f}, df_mulf(x, r));  // 1 - x r, small
    return df_add(df{r, 0.0f}, df_mulf(one_minus, r));
}

#ifdef __CUDACC__
// ---------------------------------------------------------------------------------------
// Paired FP32.  sm_100+ executes FFMA2 / FMUL2 / FADD2: one instruction, two independent
// FP32 lanes, each rounded exactly as fmaf / __fmul_rn / __fadd_rn.  On GB300 the FMA pipe
// retires paired and scalar FMAs at the same FLOP rate, so pairing does not add arithmetic
// throughput; it halves the issue slots of the paired work, and issue is what binds the
// mixed kernels.  Lanes pair independent computations: the real and imaginary parts of a
// complex entry, the two phases of a layer, the two refined roots, the two projectors.

__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// Two double-floats side by side (lane x, lane y); the operations are df_add / df_mul /
// df_fast2sum lane for lane.
struct df2 {
    float2 hi, lo;
};
__device__ __forceinline__ df2 df2_bc(df x) { return df2{bc2(x.hi), bc2(x.lo)}; }
__device__ __forceinline__ df2 df2_of(df x, df y) {
    return df2{make_float2(x.hi, y.hi), make_float2(x.lo, y.lo)};
}
__device__ __forceinline__ df df2_x(const df2& v) { return df{v.hi.x, v.lo.x}; }
__device__ __forceinline__ df df2_y(const df2& v) { return df{v.hi.y, v.lo.y}; }
__device__ __forceinline__ df2 df2_fast2sum(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    return df2{s, __fadd2_rn(b, neg2(__fadd2_rn(s, neg2(a))))};
}
__device__ __forceinline__ df2 df2_add(const df2& x, const df2& y) {
    const float2 s = __fadd2_rn(x.hi, y.hi);
    const float2 bb = __fadd2_rn(s, neg2(x.hi));
    float2 e = __fadd2_rn(__fadd2_rn(x.hi, neg2(__fadd2_rn(s, neg2(bb)))),
                          __fadd2_rn(y.hi, neg2(bb)));
    e = __fadd2_rn(e, __fadd2_rn(x.lo, y.lo));
    return df2_fast2sum(s, e);
}
__device__ __forceinline__ df2 df2_neg(const df2& x) { return df2{neg2(x.hi), neg2(x.lo)}; }
__device__ __forceinline__ df2 df2_sub(const df2& x, const df2& y) { return df2_add(x, df2_neg(y)); }
__device__ __forceinline__ df2 df2_mul(const df2& x, const df2& y) {
    const float2 p = __fmul2_rn(x.hi, y.hi);
    float2 e = __ffma2_rn(x.hi, y.hi, neg2(p));
    e = __ffma2_rn(x.hi, y.lo, __ffma2_rn(x.lo, y.hi, e));
    return df2_fast2sum(p, e);
}
#endif

// Symmetric (Loewdin-style, first order) orthonormalisation of two nearly orthonormal
// vectors: a -= (a.b)/2 b, b -= (a.b)/2 a, then both normalised.
//
// Why the FP64 fallback of the eigenvector tables needs it: the three projectors of a
// computed spectrum sum to the identity exactly whatever the root errors (they are the
// Lagrange basis polynomials of H at the computed roots), so where two levels nearly
// coincide, the errors of their two projectors cancel in S = 1 + z1 P1 + z2 P2 (z1 ~ z2).
// Unit vectors taken from each projector separately lose that cancellation: u1.u2 departs
// from 0 at first order in (root error / gap), and the reference cubic's roots of a nearly
// double root are off by ~sqrt(eps) of the spread.  Restoring orthogonality leaves only a
// rotation inside the near-degenerate plane, whose effect is multiplied by the small phase
// difference z1 - z2.
template <class T>
CP3_HD void orthonormalize_pair(T a[3], T b[3]) {
    const T h = (T)0.5 * (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    T x[3], y[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        x[i] = a[i] - h * b[i];
        y[i] = b[i] - h * a[i];
    }
    const T nx = (T)1 / sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const T ny = (T)1 / sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        a[i] = x[i] * nx;
        b[i] = y[i] * ny;
    }
}

// FP64 layer data of one (density, energy) in the rotated basis: the unit eigenvectors u1,
// u2 (P_k = u_k u_k^T, orthonormalised) and the reference's dmMatVac[k][0] = m_k - DM(0,0),
// from which the phases are formed exactly as the reference forms them.
CP3_HD void rotated_layer_f64(const OscParams* __restrict__ p, double E, double rho,
                              double u[2][3], double dmv[3]) {
    double mm[3], P[2][6];
    matter_masses_f64(p, E, rho, mm);
    rotated_projectors_f64(p, E, rho, mm, P);
    projector_vector(P[0], u[0]);
    projector_vector(P[1], u[1]);
    orthonormalize_pair(u[0], u[1]);
#pragma unroll
    for (int k = 0; k < 3; k++) dmv[k] = mm[k] - p->dm[0];
}

// The FP64 branch of the mixed eigen-solver (the reference cubic), kept out of line: inlined,
// the compiler may hoist part of it (the double conversions of E and rho) above the branch,
// and on GB300's narrow FP64 pipe even one such instruction per call costs more than the
// whole double-float path.  u[k] = the unit eigenvectors u_1, u_2, orthonormalised in FP64.
//   The fallback runs where two levels nearly meet.  There the Lagrange projectors have
// entries ~spread / gap that cancel in S = 1 + z1 P1 + z2 P2 (z1 ~ z2), and rounded to FP32
// separately they no longer do: the beam returned probabilities of 0.4-50 at the exact level
// crossing of a state without electron component (theta12 = 0 or pi/2, E ~ 0.39 GeV at
// 2.6 g/cm^3).  Orthonormal vectors give projectors of entries <= 1, exact to FP32
// rounding, and leave only a rotation inside the near-degenerate plane, which S weighs by
// the small z1 - z2.
__host__ __device__ __noinline__ inline void eigen_fallback_f64(const OscParams* __restrict__ p,
                                                                df Ed, df rhod, float uf[2][3],
                                                                float om[2][2]) {
    double Pd[2][6], omd[2], u[2][3];
    rotated_eigen_f64(p, (double)Ed.hi + (double)Ed.lo, (double)rhod.hi + (double)rhod.lo, Pd, omd);
    for (int k = 0; k < 2; k++) {
        projector_vector(Pd[k], u[k]);
        const double t = omd[k] * 0.15915494309189535;  // turns per km: omega / (2 pi)
        om[k][0] = (float)t;
        om[k][1] = (float)(t - (double)om[k][0]);
    }
    orthonormalize_pair(u[0], u[1]);
    for (int k = 0; k < 2; k++)
        for (int i = 0; i < 3; i++) uf[k][i] = (float)u[k][i];
}

// The mixed kernels' eigen-decomposition without FP64 on the common path:
//   1. V = -fac (matter potential in 2E.H units, eV^2) and the cubic's coefficients in df64;
//   2. the three roots from the trigonometric solution in FP32;
//   3. one or two Newton steps per root on the df64 polynomial (the third root from the
//      trace);
//   4. the phase rates in turns per km, omega_k / (2 pi) = 2.534 (m_k - m_0) / (2 pi E),
//      in df64 (hi, lo);
//   5. the unit eigenvectors u_1, u_2 of m_1, m_2 from the vacuum eigen-system (the
//      rank-one update below), in double-float (kDf) or FP32.
// Where two roots lie closer than 5e-3 of the spread -- tested on the FP32 starting roots
// and again on the refined ones -- the FP64 reference cubic takes over.  Below that the
// double-float Newton steps are not reliably in their quadratic regime (FP32 starting roots
// near a double root are off by ~sqrt(eps) of the spread, and Newton then converges only
// linearly, or diverges where the start sits between the pair), so neither the roots nor a
// gap test on them can be trusted there.  Physical parameters stay well above it: a scan of 2.4e6 (E, rho)
// points, 0.1-100 GeV, 0-6.6 g/cm^3 electron density, Gaussian parameter sets in both
// orderings, nu and nubar, has min gap/spread = 0.022 (100 GeV through the core); exactly
// degenerate vacuum masses (the reference's 5e-9 eV^2 degeneracy break) and the exact level
// crossings of a state without electron component (theta12 or theta13 at 0 or pi/2) are
// the cases it catches.
// E and rho arrive as float pairs (split once on the host), so the common path runs no FP64
// instruction at all -- conversions included, which issue on the narrow FP64 pipe.
//
// out[k][0..2] = u_k, the unit eigenvector with P_k = u_k u_k^T (sign arbitrary).  kDf:
// the vectors in double-float, rounded once (the eigen tables of the deep atmospheric
// chains, whose vector errors add up over the layers); else in FP32 (the beam's one layer
// per baseline).
// The common path; false where the FP64 fallback has to take over (one call site for it,
// below, so that no live range of the common path has to survive a call).
template <bool kDf>
__device__ __forceinline__ bool rotated_eigen_mixed_try(const OscParams* __restrict__ p, df Ed,
                                                        df rhod, float P[2][3], float om[2][2]) {
    // V = -fac of getMfast: +2 sqrt2 G_F N_e E for neutrinos, minus for antineutrinos.
    // (2 sqrt2 G_F) N_e comes first: constant over a beam's energies, the batched kernel
    // forms it once per tile (C3 1.2 % faster).
    const df tw = df{1.52588e-4f, -7.040322e-12f};  // kTwoRtTwoGf = hi + lo
    df V = df_mul(df_mul(tw, rhod), Ed);
    if (p->anti) V = df_neg(V);
    // det(l - H) = l^3 - c2 l^2 + c1 l - c0 with H = H0 + V e0 e0^T (OscParams::cpoly)
    const df c2 = df_add(df{p->cpolyf[0][0], p->cpolyf[0][1]}, V);
    const df c1 = df_add(df{p->cpolyf[1][0], p->cpolyf[1][1]}, df_mul(V, df{p->cpolyf[3][0], p->cpolyf[3][1]}));
    const df c0 = df_add(df{p->cpolyf[2][0], p->cpolyf[2][1]}, df_mul(V, df{p->cpolyf[4][0], p->cpolyf[4][1]}));
    // FP32 trigonometric roots of l^3 - c2 l^2 + c1 l - c0
    const float a2 = c2.hi, a1 = c1.hi, a0 = c0.hi;
    const float s = a2 * (1.0f / 3.0f);
    const float pp = fmaf(-a2, s, a1);                        // c1 - c2^2/3  (< 0)
    const float qq = fmaf(s, fmaf(-2.0f * s, s, a1), -a0);    // -(2 s^3 - s c1 + c0)
    const float mp3 = fmaxf(-pp * (1.0f / 3.0f), 1e-30f);
    // The starting roots need only ~1e-6 relative accuracy (the Newton steps below remove
    // what is left, as they remove __sincosf's), so the square root and the division take
    // the fast forms: the batched beam (8192 problems x 1e5 energies) 1 %, the 59-shell
    // 2000 x 2000 eigen table 4 % faster, every result's error unchanged.
    const float rt = mp3 * rsqrtf(mp3);
    // t = 2 sqrt(m) cos(a) solves t^3 + P t + Q = 0 when cos(3a) = -Q / (2 m^{3/2})
    const float carg = fminf(1.0f, fmaxf(-1.0f, __fdividef(-0.5f * qq, mp3 * rt)));
    const float th = acosf(carg) * (1.0f / 3.0f);
    // cos(th - 2 pi/3) = -cos(th)/2 + (sqrt(3)/2) sin(th): one sincos for both roots.  The
    // hardware approximation (absolute error ~4e-7 on [0, pi/3]) puts the starting roots
    // ~3e-7 of the spread off, no further than acos's own conditioning already does wherever
    // the gap is below ~0.2 of the spread; the Newton steps below remove either.
    float sn, cn;
    __sincosf(th, &sn, &cn);
    float l0 = fmaf(2.0f * rt, cn, s);
    float l1 = fmaf(2.0f * rt, fmaf(0.8660254f, sn, -0.5f * cn), s);
    // The fallback test, on the starting roots.  Near a double root the FP32 start is good
    // only to ~sqrt(eps) of the spread and can sit where f' vanishes between the pair; the
    // FP32 derivative is then rounding noise, the first Newton step throws the roots off by
    // a quarter of the spread, and the test on the refined roots below passes on garbage
    // (an exact level crossing of a state without electron component, theta12 = 0 or pi/2,
    // put the beam 0.6 off).  With th in [0, pi/3] the starting roots are ordered l0 >= l1 >=
    // l2, l0 - l1 = 2 sqrt3 rt sin(pi/3 - th), l1 - l2 = 2 sqrt3 rt sin(th) and the spread
    // 2 sqrt3 rt sin(th + pi/3) >= 3 rt: gap < 5e-3 spread is th (or pi/3 - th) below
    // 5e-3 sin(pi/3) = 4.33e-3.
    if (!(th > 4.33e-3f && th < 1.0471976f - 4.33e-3f)) {
        return false;
    }
    // Newton steps on both roots side by side: the residual in double-float, the derivative
    // in FP32 (its relative error, ~eps * spread / gap < 2e-5, only slows the quadratic
    // convergence by that factor).
    //   The FP32 trigonometric roots are off by ~eps * spread^2 / gap (acos near +-1), so one
    // step leaves a relative error of ~eps^2 (spread / gap)^4 in the gap: below 1e-10 while
    // gap > 0.05 spread.  The correction f / d itself needs only ~1e-6 relative accuracy
    // (it scales the remaining error, not the root), so it takes the fast divide.  The eigenvector tables of the deep atmospheric chains always take a
    // second step; the beam's projectors take it only below that gap (near the solar
    // resonance, a few per cent of a beam grid's energies).
    df2 x{make_float2(l0, l1), bc2(0.0f)};
    {
        const df2 C2 = df2_bc(c2), C1 = df2_bc(c1), C0 = df2_bc(c0);
        auto newton = [&]() {
            const df2 f = df2_sub(df2_mul(df2_add(df2_mul(df2_sub(x, C2), x), C1), x), C0);
            const float2 d = __ffma2_rn(__ffma2_rn(bc2(3.0f), x.hi, bc2(-2.0f * c2.hi)), x.hi,
                                        bc2(c1.hi));
            x = df2_sub(x, df2{make_float2(__fdividef(f.hi.x, d.x), __fdividef(f.hi.y, d.y)), bc2(0.0f)});
        };
        newton();
        bool again = kDf;
        if (!kDf) {
            const float m2 = c2.hi - x.hi.x - x.hi.y;
            const float d01 = fabsf(x.hi.x - x.hi.y), d02 = fabsf(x.hi.x - m2),
                        d12 = fabsf(x.hi.y - m2);
            again = !(fminf(d01, fminf(d02, d12)) > 0.05f * fmaxf(d01, fmaxf(d02, d12)));
        }
        if (again) newton();
    }
    df r[3] = {df2_x(x), df2_y(x), df{0.0f, 0.0f}};
    r[2] = df_sub(df_sub(c2, r[0]), r[1]);
    const float spread = fmaxf(fabsf(r[0].hi - r[1].hi), fmaxf(fabsf(r[0].hi - r[2].hi), fabsf(r[1].hi - r[2].hi)));
    const float gap = fminf(fabsf(r[0].hi - r[1].hi), fminf(fabsf(r[0].hi - r[2].hi), fabsf(r[1].hi - r[2].hi)));
    if (!(gap > 5e-3f * spread)) {
        return false;
    }
    // kLoEFac / (2 pi E): phase rates in turns per km (kLoEFac / (2 pi) = hi + lo)
    const df loe = df_mul(df{4.032986164e-01f, 9.385560773e-09f}, df_recip(Ed));
    // lane x is k = 1, lane y is k = 2; omega_k / (2 pi) = 2.534 (m_k - m_0) / (2 pi E)
    const df2 lam = df2_of(r[1], r[2]);
    const df2 w = df2_mul(df2_sub(lam, df2_bc(r[0])), df2_bc(loe));
    om[0][0] = w.hi.x;
    om[0][1] = w.lo.x;
    om[1][0] = w.hi.y;
    om[1][1] = w.lo.y;
    // Eigenvectors by the rank-one update of the vacuum system (Golub 1973; Bunch, Nielsen
    // and Sorensen 1978).  H0 = O diag(mu) O^T, so (H0 - l) u = -V (e0 . u) e0 gives
    // u = O d with d_j = a_j / (mu_j - l), a = O^T e0 (the first row of O).  Multiplied
    // through by prod_i (mu_i - l), d_j = a_j prod_{i != j} (mu_i - l): no division, and
    // finite where l meets a vacuum mass (vacuum, or a state that decouples at low density).
    // Each difference mu_i - l is formed from the double-float root before rounding to FP32
    // (hi - hi is exact or correctly rounded, the low words add ~ulp), so d is good to a few
    // ulp whatever the cancellation, and |u| = |d| (O orthogonal).
    if constexpr (kDf) {
        // The eigenvector tables feed every layer of the deep atmospheric chains, where
        // vector errors add up over the layers: on the 59-shell grid the FP32 form below
        // gave 7.5e-6 max error, double-float without the final scaling 4.5e-6, and this
        // form, rounded once after normalisation, 2.2e-6 (the same as the earlier projector
        // columns).  So the tables run the formula in double-float.
        df2 dd[3], e[3], uu[3];
#pragma unroll
        for (int i = 0; i < 3; i++) dd[i] = df2_sub(df2_bc(df{p->muf[i][0], p->muf[i][1]}), lam);
        auto o = [&](int i, int j) { return df2_bc(df{p->of[i][j], p->oflo[i][j]}); };
        e[0] = df2_mul(o(0, 0), df2_mul(dd[1], dd[2]));
        e[1] = df2_mul(o(0, 1), df2_mul(dd[0], dd[2]));
        e[2] = df2_mul(o(0, 2), df2_mul(dd[0], dd[1]));
#pragma unroll
        for (int i = 0; i < 3; i++)
            uu[i] = df2_add(df2_add(df2_mul(o(i, 0), e[0]), df2_mul(o(i, 1), e[1])), df2_mul(o(i, 2), e[2]));
        const df2 nn = df2_add(df2_add(df2_mul(e[0], e[0]), df2_mul(e[1], e[1])), df2_mul(e[2], e[2]));
        const float s2 = spread * spread;
        if (!(fminf(nn.hi.x, nn.hi.y) > 1e-16f * (s2 * s2))) {  // see the FP32 branch below
            return false;
        }
        // 1 / sqrt(n) in double-float: the float estimate r, then one Newton step on the
        // exact residual 1 - n r^2 (r^2 and n.hi r^2 through TwoProduct); the vector is
        // scaled in double-float and rounded once (1/2 ulp, as the tables were before)
        const float2 r = make_float2(rsqrtf(nn.hi.x), rsqrtf(nn.hi.y));
        const float2 r2 = __fmul2_rn(r, r), r2e = __ffma2_rn(r, r, neg2(r2));
        const float2 q = __fmul2_rn(nn.hi, r2), qe = __ffma2_rn(nn.hi, r2, neg2(q));
        float2 res = __fadd2_rn(bc2(1.0f), neg2(q));  // exact: q is within an ulp or two of 1
        res = __fadd2_rn(res, neg2(__ffma2_rn(nn.lo, r2, __ffma2_rn(nn.hi, r2e, qe))));
        const df2 rn = df2_fast2sum(r, __fmul2_rn(__fmul2_rn(r, bc2(0.5f)), res));
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const df2 v = df2_mul(uu[i], rn);
            const float2 f = __fadd2_rn(v.hi, v.lo);
            P[0][i] = f.x;
            P[1][i] = f.y;
        }
        return true;
    } else {
        float2 dl[3];
#pragma unroll
        for (int i = 0; i < 3; i++)
            dl[i] = __fadd2_rn(__fadd2_rn(bc2(p->muf[i][0]), neg2(lam.hi)),
                               __fadd2_rn(bc2(p->muf[i][1]), neg2(lam.lo)));
        float2 d[3];
        d[0] = __fmul2_rn(bc2(p->of[0][0]), __fmul2_rn(dl[1], dl[2]));
        d[1] = __fmul2_rn(bc2(p->of[0][1]), __fmul2_rn(dl[0], dl[2]));
        d[2] = __fmul2_rn(bc2(p->of[0][2]), __fmul2_rn(dl[0], dl[1]));
        float2 u[3];
#pragma unroll
        for (int i = 0; i < 3; i++)
            u[i] = __ffma2_rn(bc2(p->of[i][2]), d[2],
                              __ffma2_rn(bc2(p->of[i][1]), d[1], __fmul2_rn(bc2(p->of[i][0]), d[0])));
        const float2 n = __ffma2_rn(d[2], d[2], __ffma2_rn(d[1], d[1], __fmul2_rn(d[0], d[0])));
        // |d|^2 ~ spread^4 except where the formula has no content: a vacuum mass shared by two
        // states (a degenerate splitting) or a state with no electron component (a_j = 0, e.g.
        // theta13 = 0), where d vanishes with l - mu_j.  Those parameter sets take the FP64
        // reference path; physical ones stay above 1e-12 spread^4.
        const float s2 = spread * spread;
        if (!(fminf(n.x, n.y) > 1e-16f * (s2 * s2))) {
            return false;
        }
        // the unit vectors u / |d|, good to a few ulp: the beam's one layer per baseline needs
        // no more
        const float2 r = make_float2(rsqrtf(n.x), rsqrtf(n.y));
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float2 v = __fmul2_rn(u[i], r);
            P[0][i] = v.x;
            P[1][i] = v.y;
        }
        return true;
    }
}

template <bool kDf>
__device__ __forceinline__ void rotated_eigen_mixed_t(const OscParams* __restrict__ p, df Ed,
                                                      df rhod, float u[2][3], float om[2][2]) {
    if (!rotated_eigen_mixed_try<kDf>(p, Ed, rhod, u, om)) eigen_fallback_f64(p, Ed, rhod, u, om);
}

// Unit eigenvectors u1, u2 (P_k = u_k u_k^T) and phase rates; the vectors in double-float,
// rounded once (the eigen tables).
__device__ __forceinline__ void rotated_eigen_vectors(const OscParams* __restrict__ p, df Ed,
                                                      df rhod, float u[2][3], float om[2][2]) {
    rotated_eigen_mixed_t<true>(p, Ed, rhod, u, om);
}
// The same with the vectors in FP32 (the beam).
__device__ __forceinline__ void rotated_eigen_vectors_fp32(const OscParams* __restrict__ p, df Ed,
                                                           df rhod, float u[2][3], float om[2][2]) {
    rotated_eigen_mixed_t<false>(p, Ed, rhod, u, om);
}
__device__ __forceinline__ void rotated_eigen_vectors_fp32(const OscParams* __restrict__ p, double E,
                                                           double rho, float u[2][3], float om[2][2]) {
    rotated_eigen_mixed_t<false>(p, df_from(E), df_from(rho), u, om);
}

CP3_HD cf cmulf(cf a, cf b) {
    return cf{fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re)};
}

}  // namespace cp3

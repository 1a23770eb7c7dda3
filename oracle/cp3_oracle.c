/*
 * cp3_oracle.c -- CPU oracle for the Barger propagation path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of CUDAProb3++'s FP64 CPU propagation
 * (AtmosCpuPropagator<double>::calculateProbabilities and
 * BeamCpuPropagator<double>::calculateProbabilities).  Every function names the
 * reference function and file:line it restates.  The arithmetic of each formula is kept
 * in the reference's evaluation order, so that this file reproduces the reference's
 * rounding and not only its mathematics; the fixtures in tests/golden/ (made by the
 * reference's own headers, see oracle/Makefile target `ref`) pin it.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this file.
 * The product library never links it.
 */
#include "cp3_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constants.hpp:26-50 */
#define K_TWORTTWOGF 1.52588e-4
#define K_KM2CM 1.0e5
#define K_REARTH 6371.0
#define K_REARTHCM (K_REARTH * K_KM2CM)
#define K_DENSITY_CONVERT 0.5
#define K_EPSILON 1e-6
/* (1/2)*(1/(hbar c)) in GeV/(eV^2 km): physics.hpp:443 and :524 */
#define K_LOEFAC 2.534

typedef struct {
    double re, im;
} cx;

/* Everything the reference keeps in its process-global parameter store
 * (physics.hpp:115-125): U, DM, AXFAC, mass order. Here it is a value. */
typedef struct {
    cx U[9];           /* U(i,j) = U[i*3+j] */
    double dm[9];      /* DM(i,j) = dm[i*3+j] */
    double axfac[324]; /* AXFAC(a,b,c,d,e) = axfac[(((a*3+b)*3+c)*3+d)*4+e] */
    int order[3];
} osc_state;

#define UU(s, i, j) ((s)->U[(i) * 3 + (j)])
#define DMM(s, i, j) ((s)->dm[(i) * 3 + (j)])
#define AXF(s, a, b, c, d, e) ((s)->axfac[((((a) * 3 + (b)) * 3 + (c)) * 3 + (d)) * 4 + (e)])

/* Propagator::setMNSMatrix (propagator.hpp:148-183): PDG parametrisation, dcp sign
 * flipped when kNuType < 0. */
static void build_pmns(osc_state* s, const orc_mixing* m) {
    double dcp = m->dcp;
    if (m->knutype < 0) dcp *= -1;
    const double s12 = sin(m->theta12), s13 = sin(m->theta13), s23 = sin(m->theta23);
    const double c12 = cos(m->theta12), c13 = cos(m->theta13), c23 = cos(m->theta23);
    const double sd = sin(dcp), cd = cos(dcp);
    UU(s, 0, 0).re = c12 * c13;                      UU(s, 0, 0).im = 0.0;
    UU(s, 0, 1).re = s12 * c13;                      UU(s, 0, 1).im = 0.0;
    UU(s, 0, 2).re = s13 * cd;                       UU(s, 0, 2).im = -s13 * sd;
    UU(s, 1, 0).re = -s12 * c23 - c12 * s23 * s13 * cd; UU(s, 1, 0).im = -c12 * s23 * s13 * sd;
    UU(s, 1, 1).re = c12 * c23 - s12 * s23 * s13 * cd;  UU(s, 1, 1).im = -s12 * s23 * s13 * sd;
    UU(s, 1, 2).re = s23 * c13;                      UU(s, 1, 2).im = 0.0;
    UU(s, 2, 0).re = s12 * s23 - c12 * c23 * s13 * cd;  UU(s, 2, 0).im = -c12 * c23 * s13 * sd;
    UU(s, 2, 1).re = -c12 * s23 - s12 * c23 * s13 * cd; UU(s, 2, 1).im = -s12 * c23 * s13 * sd;
    UU(s, 2, 2).re = c23 * c13;                      UU(s, 2, 2).im = 0.0;
}

/* Propagator::setNeutrinoMasses (propagator.hpp:188-209): vacuum masses relative to m1,
 * with the 5e-9 eV^2 degeneracy break. */
static void build_mass_matrix(osc_state* s, double dm12sq, double dm23sq) {
    double mv[3] = {0.0, dm12sq, dm12sq + dm23sq};
    const double delta = 5.0e-9;
    if (dm12sq == 0.0) mv[0] -= delta;
    if (dm23sq == 0.0) mv[2] += delta;
    for (int i = 0; i < 3; i++) DMM(s, i, i) = 0.0;
    DMM(s, 0, 1) = mv[0] - mv[1];
    DMM(s, 1, 0) = -DMM(s, 0, 1);
    DMM(s, 0, 2) = mv[0] - mv[2];
    DMM(s, 2, 0) = -DMM(s, 0, 2);
    DMM(s, 1, 2) = mv[1] - mv[2];
    DMM(s, 2, 1) = -DMM(s, 1, 2);
}

/* physics::setMixMatrix_host (physics.hpp:158-174): U-bilinears used by getA. */
static void build_axfac(osc_state* s) {
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const cx a = UU(s, n, i), b = UU(s, m, j);
                    AXF(s, n, m, i, j, 0) = a.re * b.re + a.im * b.im;
                    AXF(s, n, m, i, j, 1) = a.re * b.im - a.im * b.re;
                    AXF(s, n, m, i, j, 2) = a.im * b.im + a.re * b.re;
                    AXF(s, n, m, i, j, 3) = a.im * b.re - a.re * b.im;
                }
}

/* physics::prepare_getMfast (physics.hpp:198-252): solve the vacuum cubic the same way as
 * the matter one and record which root reproduces each vacuum state. */
static void build_mass_order(osc_state* s) {
    const double alphaV = DMM(s, 0, 1) + DMM(s, 0, 2);
    const double betaV = DMM(s, 0, 1) * DMM(s, 0, 2);
    const double gammaV = 0.0;
    double tmpV = alphaV * alphaV - 3.0 * betaV;
    double argV = (2.0 * alphaV * alphaV * alphaV - 9.0 * alphaV * betaV + 27.0 * gammaV) /
                  (2.0 * sqrt(tmpV * tmpV * tmpV));
    if (fabs(argV) > 1.0) argV = argV / fabs(argV);
    const double th0 = acos(argV) / 3.0;
    const double th1 = th0 - (2.0 * M_PI / 3.0);
    const double th2 = th0 + (2.0 * M_PI / 3.0);
    double root[3];
    root[0] = root[1] = root[2] = -(2.0 / 3.0) * sqrt(tmpV);
    root[0] *= cos(th0);
    root[1] *= cos(th1);
    root[2] *= cos(th2);
    tmpV = DMM(s, 0, 0) - alphaV / 3.0;
    for (int k = 0; k < 3; k++) root[k] += tmpV;
    for (int i = 0; i < 3; i++) {
        double best = fabs(DMM(s, i, 0) - root[0]);
        int k = 0;
        for (int j = 1; j < 3; j++) {
            const double d = fabs(DMM(s, i, 0) - root[j]);
            if (d < best) {
                k = j;
                best = d;
            }
        }
        s->order[i] = k;
    }
}

static void osc_setup(osc_state* s, const orc_mixing* m) {
    build_pmns(s, m);
    build_mass_matrix(s, m->dm12sq, m->dm23sq);
    build_axfac(s);
    build_mass_order(s);
}

/* physics::getMfast (physics.hpp:267-340): matter eigenvalues (Barger et al. eq. 21-22),
 * returned as mass-mass and mass-vacuum difference matrices. */
static void matter_masses(const osc_state* s, double E, double rho, int anti,
                          double dMM[3][3], double dMV[3][3]) {
    const double fac = anti ? K_TWORTTWOGF * E * rho : -K_TWORTTWOGF * E * rho;
    const double alpha = fac + DMM(s, 0, 1) + DMM(s, 0, 2);
    const double beta = DMM(s, 0, 1) * DMM(s, 0, 2) +
                        fac * (DMM(s, 0, 1) * (1.0 - UU(s, 0, 1).re * UU(s, 0, 1).re -
                                               UU(s, 0, 1).im * UU(s, 0, 1).im) +
                               DMM(s, 0, 2) * (1.0 - UU(s, 0, 2).re * UU(s, 0, 2).re -
                                               UU(s, 0, 2).im * UU(s, 0, 2).im));
    const double gamma = fac * DMM(s, 0, 1) * DMM(s, 0, 2) *
                         (UU(s, 0, 0).re * UU(s, 0, 0).re + UU(s, 0, 0).im * UU(s, 0, 0).im);
    const double tmp = alpha * alpha - 3.0 * beta < 0 ? 0 : alpha * alpha - 3.0 * beta;
    const double argtmp = (2.0 * alpha * alpha * alpha - 9.0 * alpha * beta + 27.0 * gamma) /
                          (2.0 * sqrt(tmp * tmp * tmp));
    const double arg = fabs(argtmp) > 1.0 ? argtmp / fabs(argtmp) : argtmp;
    const double th0 = acos(arg) / 3.0;
    const double th1 = th0 - (2.0 * M_PI / 3.0);
    const double th2 = th0 + (2.0 * M_PI / 3.0);
    double root[3];
    root[0] = -(2.0 / 3.0) * sqrt(tmp);
    root[1] = -(2.0 / 3.0) * sqrt(tmp);
    root[2] = -(2.0 / 3.0) * sqrt(tmp);
    root[0] *= cos(th0);
    root[1] *= cos(th1);
    root[2] *= cos(th2);
    const double shift = DMM(s, 0, 0) - alpha / 3.0;
    for (int k = 0; k < 3; k++) root[k] += shift;
    double mm[3];
    for (int i = 0; i < 3; i++) mm[i] = root[s->order[i]];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            dMM[i][j] = mm[i] - mm[j];
            dMV[i][j] = mm[i] - DMM(s, j, 0);
        }
}

/* physics::get_product (physics.hpp:345-430): in the mass basis, the products
 * (2EH - M_a)(2EH - M_b) / (dm_ka dm_kb) for the three expansion indices k. */
static void spectral_products(const osc_state* s, double E, double rho, int anti,
                              const double dMV[3][3], const double dMM[3][3],
                              cx prod[3][3][3]) {
    const double fac = anti ? K_TWORTTWOGF * E * rho : -K_TWORTTWOGF * E * rho;
    cx h[3][3][3]; /* h[n][m][j] = (2EH - M_j)_{nm} */
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++) {
            const cx a = UU(s, 0, n), b = UU(s, 0, m);
            const double re = -fac * (a.re * b.re + a.im * b.im);
            const double im = -fac * (a.re * b.im - a.im * b.re);
            for (int j = 0; j < 3; j++) {
                h[n][m][j].re = re;
                h[n][m][j].im = im;
            }
        }
    for (int j = 0; j < 3; j++) {
        h[0][0][j].re -= dMV[j][0];
        h[1][1][j].re -= dMV[j][1];
        h[2][2][j].re -= dMV[j][2];
    }
    /* expansion index k pairs the two other roots: k=0 <- (1,2), k=1 <- (2,0), k=2 <- (0,1) */
    static const int first[3] = {1, 2, 0};
    static const int second[3] = {2, 0, 1};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            for (int k = 0; k < 3; k++) prod[i][j][k].re = prod[i][j][k].im = 0;
            for (int q = 0; q < 3; q++)
                for (int k = 0; k < 3; k++) {
                    const cx x = h[i][q][first[k]], y = h[q][j][second[k]];
                    prod[i][j][k].re += x.re * y.re - x.im * y.im;
                    prod[i][j][k].im += x.re * y.im + x.im * y.re;
                }
            const double d0 = dMM[0][1] * dMM[0][2];
            const double d1 = dMM[1][2] * dMM[1][0];
            const double d2 = dMM[2][0] * dMM[2][1];
            prod[i][j][0].re /= d0;
            prod[i][j][0].im /= d0;
            prod[i][j][1].re /= d1;
            prod[i][j][1].im /= d1;
            prod[i][j][2].re /= d2;
            prod[i][j][2].im /= d2;
        }
}

/* physics::getArg (physics.hpp:439-450), phase_offset = 0. */
static void expansion_phases(double L, double E, const double dMV[3][3], double arg[3]) {
    for (int k = 0; k < 3; k++) arg[k] = -K_LOEFAC * dMV[k][0] * L / E;
}

/* physics::getC (physics.hpp:459-514): C_k = U . product_k . U^dagger (flavour basis). */
static void flavour_projectors(const osc_state* s, const cx prod[3][3][3], cx C[3][3][3]) {
    for (int k = 0; k < 3; k++)
        for (int a = 0; a < 3; a++) {
            double RR[3] = {0, 0, 0}, RI[3] = {0, 0, 0}, IR[3] = {0, 0, 0}, II[3] = {0, 0, 0};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    RR[j] += UU(s, a, i).re * prod[i][j][k].re;
                    RI[j] += UU(s, a, i).re * prod[i][j][k].im;
                    IR[j] += UU(s, a, i).im * prod[i][j][k].re;
                    II[j] += UU(s, a, i).im * prod[i][j][k].im;
                }
            for (int b = 0; b < 3; b++) {
                double re = 0., im = 0.;
                for (int j = 0; j < 3; j++) {
                    re += RR[j] * UU(s, b, j).re;
                    re += RI[j] * UU(s, b, j).im;
                    re += IR[j] * UU(s, b, j).im;
                    re -= II[j] * UU(s, b, j).re;
                    im += II[j] * UU(s, b, j).im;
                    im += IR[j] * UU(s, b, j).re;
                    im += RI[j] * UU(s, b, j).re;
                    im -= RR[j] * UU(s, b, j).im;
                }
                C[k][a][b].re = re;
                C[k][a][b].im = im;
            }
        }
}

/* math::multiply_phase_matrix (math.hpp:59-75): B += exp(i phase) A. */
static void add_phased(double phase, const cx A[3][3], cx B[3][3]) {
    const double sn = sin(phase), cs = cos(phase);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            B[i][j].re += cs * A[i][j].re - sn * A[i][j].im;
            B[i][j].im += cs * A[i][j].im + sn * A[i][j].re;
        }
}

/* math::multiply_complex_matrix (math.hpp:84-96) followed by copy: R = A . B. */
static void matmul(const cx A[3][3], const cx B[3][3], cx R[3][3]) {
    cx t[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            t[i][j].re = 0;
            t[i][j].im = 0;
            for (int k = 0; k < 3; k++) {
                t[i][j].re += A[i][k].re * B[k][j].re - A[i][k].im * B[k][j].im;
                t[i][j].im += A[i][k].im * B[k][j].re + A[i][k].re * B[k][j].im;
            }
        }
    memcpy(R, t, sizeof(t));
}

/* physics::getA (physics.hpp:516-598): A = U (sum_k e^{i arg_k} product_k) U^dagger via AXFAC. */
static void beam_amplitude(const osc_state* s, double L, double E, const double dMV[3][3],
                           const cx prod[3][3][3], cx A[3][3]) {
    cx X[3][3];
    memset(X, 0, sizeof(X));
    for (int k = 0; k < 3; k++) {
        const double arg = -K_LOEFAC * dMV[k][0] * L / E;
        const double sn = sin(arg), cs = cos(arg);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                X[i][j].re += cs * prod[i][j][k].re - sn * prod[i][j][k].im;
                X[i][j].im += cs * prod[i][j][k].im + sn * prod[i][j][k].re;
            }
    }
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++) {
            A[n][m].re = 0;
            A[n][m].im = 0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    A[n][m].re += AXF(s, n, m, i, j, 0) * X[i][j].re + AXF(s, n, m, i, j, 1) * X[i][j].im;
                    A[n][m].im += AXF(s, n, m, i, j, 2) * X[i][j].im + AXF(s, n, m, i, j, 3) * X[i][j].re;
                }
        }
}

/* physics::getDensityOfLayer (physics.hpp:634-646). */
static double layer_density(const orc_earth* e, int layer, int maxl) {
    if (layer == 0) return 0.0;
    const int i = layer <= maxl ? layer - 1 : 2 * maxl - layer - 1;
    return e->rhos[i] * e->yps[i];
}

/* physics::getDensityOfLayerPoly (physics.hpp:651-739): path average of a r^2 + b r + c
 * over the segment, times Ye. distance_cm is the segment length. */
static double layer_density_poly(const orc_earth* e, double cosz, int layer, int maxl,
                                 double distance_cm) {
    if (cosz >= 0) return 0;
    if (layer == 0) return 0;
    const int i = layer <= maxl ? layer - 1 : 2 * maxl - layer - 1;
    const double* r = e->radii;
    const double Rmin2 = pow(K_REARTH, 2) * (1 - pow(cosz, 2));
    const double Rmax2 = pow(r[i], 2);
    const double dist = sqrt(Rmax2 - Rmin2);
    if (Rmin2 == 0) {
        /* radial trajectory: plain radial average over the shell */
        const double hi = e->as[i] * pow(r[i], 3) / 3. + e->bs[i] * pow(r[i], 2) / 2. + e->cs[i] * r[i];
        const double lo = e->as[i] * pow(r[i + 1], 3) / 3. + e->bs[i] * pow(r[i + 1], 2) / 2. +
                          e->cs[i] * r[i + 1];
        double density = hi - lo;
        density /= (r[i] - r[i + 1]);
        return density * e->yps[i];
    }
    /* along the path R(t)^2 = a t^2 + b t + c, t in km from the shell's outer edge */
    const double a = 1.0, b = -2 * dist, c = Rmax2;
    const double t2 = distance_cm / K_KM2CM;
    const double t1 = 0.;
    const double sq_p = a * pow(t2, 3) / 3. + b * pow(t2, 2) / 2. + c * t2;
    const double sq_m = a * pow(t1, 3) / 3. + b * pow(t1, 2) / 2. + c * t1;
    const double sq = sq_p - sq_m;
    const double lp1 = (b + 2. * a * t2) * sqrt(c + t2 * (b + a * t2)) / (4. * a);
    const double lm1 = (b + 2. * a * t1) * sqrt(c + t1 * (b + a * t1)) / (4. * a);
    const double lp2 = (b * b - 4. * a * c) *
                       log(b + 2. * a * t2 + 2. * sqrt(a) * sqrt(c + t2 * (b + a * t2))) /
                       (8. * pow(a, 3. / 2.));
    const double lm2 = (b * b - 4. * a * c) *
                       log(b + 2. * a * t1 + 2. * sqrt(a) * sqrt(c + t1 * (b + a * t1))) /
                       (8. * pow(a, 3. / 2.));
    const double lin = (lp1 - lp2) - (lm1 - lm2);
    const double con = t2 - t1;
    const double density = (e->as[i] * sq + e->bs[i] * lin + e->cs[i] * con) / (t2 - t1);
    return density * e->yps[i];
}

/* physics::getTraversedDistanceOfLayer (physics.hpp:745-787); result in cm.
 * The innermost crossed shell reads only its own radius (the reference also evaluates the
 * next radius there, which needs the r=0 row; the value is discarded either way). */
static double layer_distance(const double* radii, int layer, int maxl, double path_cm,
                             double earth_cm, double cosz) {
    if (cosz >= 0) return path_cm;
    if (layer == 0) return path_cm - earth_cm;
    const int i = layer <= maxl ? layer - 1 : 2 * maxl - layer - 1;
    const double R2min = K_REARTH * K_REARTH * (1 - cosz * cosz);
    double cross_this = 2.0 * sqrt(radii[i] * radii[i] - R2min);
    if (sqrt(R2min) > radii[i]) cross_this = 0;
    if (i < maxl - 1) {
        double cross_next = 2.0 * sqrt(radii[i + 1] * radii[i + 1] - R2min);
        if (sqrt(R2min) > radii[i + 1]) cross_next = 0;
        return 0.5 * (cross_this - cross_next) * K_KM2CM;
    }
    return cross_this * K_KM2CM;
}

/* PathLength of calculate_atmos (physics.hpp:897-898), cm. */
static double path_length_cm(double h_cm, double cosz) {
    return sqrt((K_REARTHCM + h_cm) * (K_REARTHCM + h_cm) -
                (K_REARTHCM * K_REARTHCM) * (1 - cosz * cosz)) -
           K_REARTHCM * cosz;
}

/* math::defined_sinc (math.hpp:49-55).  The reference tests `abs(A) >= Epsilon()` with an
 * unqualified abs on a double, which binds to int abs(int): the argument is truncated, so
 * the Taylor branch is taken for every |x| < 1 (checked against the reference build).
 * Restated as the reference behaves: truncation to an int of magnitude >= 1e-6 is the
 * same test as |x| >= 1. */
static double sinc_defined(double x) {
    if (fabs(x) >= 1.0) return sin(x) / x;
    return 1.0 - x * x / 6. + x * x * x * x / 120.;
}

int orc_flip_model(int n, const double* radii, const double* c1, const double* c2,
                   const double* c3, const double* c4, double* radii_out, double* c1_out,
                   double* c2_out, double* c3_out, double* c4_out) {
    /* AtmosCpuPropagator::setDensity (atmoscpupropagator.hpp:116-170, 181-242) */
    if (n <= 0) return ORC_BAD_SIZE;
    int flip = 0;
    if (n >= 2) {
        const int sign = radii[1] - radii[0] > 0 ? 1 : -1;
        for (int i = 1; i < n; i++)
            if ((radii[i] - radii[i - 1]) * sign < 0) return ORC_BAD_ORDER;
        if (sign == 1) flip = 1;
    }
    const double* src[5] = {radii, c1, c2, c3, c4};
    double* dst[5] = {radii_out, c1_out, c2_out, c3_out, c4_out};
    for (int v = 0; v < 5; v++) {
        if (!src[v] || !dst[v]) continue;
        for (int i = 0; i < n; i++) dst[v][i] = src[v][flip ? n - 1 - i : i];
    }
    return ORC_OK;
}

int orc_max_layers(const double* radii, int n_radii, const double* cosines, int nc, int limit,
                   int* maxlayers) {
    /* coslimit: atmoscpupropagator.hpp:160-167; count: :431-444 */
    double* lim = (double*)malloc(sizeof(double) * (size_t)(n_radii > 0 ? n_radii : 1));
    if (!lim) return ORC_BAD_ARGUMENT;
    for (int i = 0; i < n_radii; i++) {
        double x = -1 * sqrt(1 - (radii[i] * radii[i] / (K_REARTH * K_REARTH)));
        if (i == 0) x = 0;
        lim[i] = x;
    }
    int rc = ORC_OK;
    for (int ic = 0; ic < nc; ic++) {
        int cnt = 0;
        for (int i = 0; i < n_radii; i++)
            if (cosines[ic] < lim[i]) cnt++;
        if (cnt > limit) rc = ORC_LAYER_LIMIT;
        maxlayers[ic] = cnt;
    }
    free(lim);
    return rc;
}

int orc_trajectory(const orc_earth* earth, double cosz, double prod_height_km, int M,
                   double* seg_len_km, double* seg_rho) {
    const double h_cm = prod_height_km * 100000.0;
    const double earth_cm = -2.0 * cosz * K_REARTHCM;
    const double path_cm = path_length_cm(h_cm, cosz);
    for (int l = 0; l <= M; l++) {
        const double d = layer_distance(earth->radii, l, M, path_cm, earth_cm, cosz);
        seg_len_km[l] = d / K_KM2CM;
        seg_rho[l] = earth->poly ? layer_density_poly(earth, cosz, l, M, d) : layer_density(earth, l, M);
    }
    return M;
}

/* physics::calculate_atmos (physics.hpp:789-1150), host branch: OpenMP over cosines. */
int orc_atmos(const orc_mixing* mix, int anti, const double* cosines, int nc,
              const double* energies, int ne, const orc_earth* earth, double prod_height_km,
              int avg, int n_ph_bins, const double* ph_prob, const double* ph_edges,
              int layer_limit, int nthreads, double* out) {
    if (nc < 0 || ne < 0 || !earth || earth->n <= 0) return ORC_BAD_SIZE;
    if (avg && (n_ph_bins < 1 || !ph_prob || !ph_edges)) return ORC_BAD_ARGUMENT;
    osc_state st;
    osc_setup(&st, mix);
    int* maxl = (int*)malloc(sizeof(int) * (size_t)(nc > 0 ? nc : 1));
    if (!maxl) return ORC_BAD_ARGUMENT;
    const int rc = orc_max_layers(earth->radii, earth->n, cosines, nc, layer_limit, maxl);
    if (rc != ORC_OK) {
        free(maxl);
        return rc;
    }
    /* setProductionHeight stores heightKM * 100000.0 (atmoscpupropagator.hpp:390) */
    const double h_cm = prod_height_km * 100000.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (int ic = 0; ic < nc; ic++) {
        const double cosz = cosines[ic];
        const double earth_cm = -2.0 * cosz * K_REARTHCM;
        const int M = maxl[ic];
        for (int ie = 0; ie < ne; ie++) {
            const double E = energies[ie];
            cx fin[3][3], mantle[3][3], T[3][3], C[3][3][3], Catm[3][3][3];
            double arg[3], darg0[3] = {0, 0, 0}, dMM[3][3], dMV[3][3];
            cx prod[3][3][3];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    mantle[i][j].re = i == j ? 1.0 : 0.0;
                    mantle[i][j].im = 0.0;
                }
            const double path_cm = path_length_cm(h_cm, cosz);
            for (int l = 0; l <= M; l++) {
                const double dist = layer_distance(earth->radii, l, M, path_cm, earth_cm, cosz);
                const double rho = earth->poly ? layer_density_poly(earth, cosz, l, M, dist)
                                               : layer_density(earth, l, M);
                /* get_transition_matrix_expansion (physics.hpp:620-629) */
                matter_masses(&st, E, rho, anti, dMM, dMV);
                expansion_phases(dist / K_KM2CM, E, dMV, arg);
                spectral_products(&st, E, rho, anti, dMV, dMM, prod);
                flavour_projectors(&st, prod, C);
                memset(T, 0, sizeof(T));
                for (int k = 0; k < 3; k++) add_phased(arg[k], C[k], T);
                if (l == 0) {
                    memcpy(fin, T, sizeof(T));
                    memcpy(Catm, C, sizeof(C));
                    if (dist != 0.)
                        for (int k = 0; k < 3; k++) darg0[k] = arg[k] / dist;
                } else if (l < M) {
                    matmul(T, fin, fin);
                    matmul(mantle, T, mantle);
                } else {
                    matmul(T, fin, fin);
                }
            }
            matmul(mantle, fin, fin);

            /* production-height shift factors (physics.hpp:997-1079), [k][k'][initial flavour] */
            cx shift[3][3][3];
            memset(shift, 0, sizeof(shift));
            if (avg) {
                for (int a = 0; a < 3; a++)
                    for (int f = 0; f < 3; f++) shift[a][a][f].re = 1.0;
                double dL[64];
                const int nb = n_ph_bins;
                for (int p = 0; p < nb + 1 && p < 64; p++) {
                    const double hcm = K_KM2CM * ph_edges[p];
                    dL[p] = path_length_cm(hcm, cosz) - path_cm;
                }
                for (int p = 0; p < nb; p++) {
                    const double h0 = dL[p], h1 = dL[p + 1];
                    const double hm = (h1 + h0) / 2., hw = (h1 - h0);
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < a; b++) {
                            const double d = darg0[a] - darg0[b];
                            const double sarg = 0.5 * d * hw;
                            const double fre = sinc_defined(sarg) * cos(d * hm);
                            const double fim = sinc_defined(sarg) * sin(d * hm);
                            for (int f = 0; f < 3; f++) {
                                const size_t idx = (size_t)anti * 3 * ne * nc * nb +
                                                   (size_t)f * ne * nc * nb +
                                                   (size_t)ie * nc * nb + (size_t)ic * nb + p;
                                const double w = ph_prob[idx];
                                shift[a][b][f].re += w * fre;
                                shift[a][b][f].im += w * fim;
                                shift[b][a][f].re += w * fre;
                                shift[b][a][f].im -= w * fim;
                            }
                        }
                }
            } else {
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < a; b++)
                        for (int f = 0; f < 3; f++) {
                            shift[a][b][f].re = 1.0;
                            shift[a][b][f].im = 0.;
                        }
            }

            /* probabilities from fin . C_atm[k] (physics.hpp:1102-1130) */
            cx P[3][3][3];
            for (int k = 0; k < 3; k++) {
                memset(P[k], 0, sizeof(P[k]));
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int q = 0; q < 3; q++) {
                            P[k][i][j].re += fin[i][q].re * Catm[k][q][j].re - fin[i][q].im * Catm[k][q][j].im;
                            P[k][i][j].im += fin[i][q].im * Catm[k][q][j].re + fin[i][q].re * Catm[k][q][j].im;
                        }
            }
            double prob[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int k = 0; k < 3; k++) {
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++)
                        prob[i][j] += P[k][i][j].re * P[k][i][j].re + P[k][i][j].im * P[k][i][j].im;
                for (int q = 0; q < k; q++)
                    for (int j = 0; j < 3; j++)
                        for (int i = 0; i < 3; i++)
                            prob[i][j] += 2. * P[q][i][j].re * P[k][i][j].re * shift[k][q][j].re +
                                          2. * P[q][i][j].im * P[k][i][j].im * shift[k][q][j].re +
                                          2. * P[q][i][j].im * P[k][i][j].re * shift[k][q][j].im -
                                          2. * P[q][i][j].re * P[k][i][j].im * shift[k][q][j].im;
            }
            double* o = out + ((size_t)ic * ne + ie) * 9;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) o[i * 3 + j] = prob[j][i];
        }
    }
    free(maxl);
    return ORC_OK;
}

/* physics::calculate_beam (physics.hpp:1153-1260), host branch: OpenMP over energies. */
int orc_beam(const orc_mixing* mix, int anti, const double* energies, int ne, double rho,
             double path_km, int nthreads, double* out) {
    if (ne < 0) return ORC_BAD_SIZE;
    osc_state st;
    osc_setup(&st, mix);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for
#endif
    for (int ie = 0; ie < ne; ie++) {
        const double E = energies[ie];
        double dMM[3][3], dMV[3][3];
        cx prod[3][3][3], A[3][3];
        const double rho_e = rho * K_DENSITY_CONVERT;
        matter_masses(&st, E, rho_e, anti, dMM, dMV);
        spectral_products(&st, E, rho_e, anti, dMV, dMM, prod);
        beam_amplitude(&st, path_km, E, dMV, prod, A);
        double* o = out + (size_t)ie * 9;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) o[i * 3 + j] = A[j][i].re * A[j][i].re + A[j][i].im * A[j][i].im;
    }
    return ORC_OK;
}

void orc_transition_matrix(const orc_mixing* mix, int anti, double E, double rho_e, double L_km,
                           double* A18) {
    osc_state st;
    osc_setup(&st, mix);
    double dMM[3][3], dMV[3][3];
    cx prod[3][3][3], A[3][3];
    matter_masses(&st, E, rho_e, anti, dMM, dMV);
    spectral_products(&st, E, rho_e, anti, dMV, dMM, prod);
    beam_amplitude(&st, L_km, E, dMV, prod, A);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            A18[(i * 3 + j) * 2] = A[i][j].re;
            A18[(i * 3 + j) * 2 + 1] = A[i][j].im;
        }
}

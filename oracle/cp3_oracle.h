/*
 * cp3_oracle.h -- CPU oracle for the Barger propagation path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of CUDAProb3++'s CPU propagators
 * (AtmosCpuPropagator<double>, BeamCpuPropagator<double>). It exists so that the
 * test-suite, the smoke check and the CPU baseline of bench.py have an independent
 * FP64 checker. The product library (cudaprob3_gb300) never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself: the fixtures in
 * tests/golden/ were produced by the reference's own headers compiled by
 * oracle/Makefile (target `ref`), and tests/test_oracle.py checks this file against them.
 */
#ifndef CP3_ORACLE_H
#define CP3_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Oscillation parameters exactly as a user hands them to the reference
 * (Propagator::setMNSMatrix, propagator.hpp:148; setNeutrinoMasses, propagator.hpp:188). */
typedef struct {
    double theta12, theta13, theta23, dcp; /* radians */
    int knutype;                           /* < 0 flips the sign of dcp */
    double dm12sq, dm23sq;                 /* eV^2; dm23sq = m3^2 - m2^2 */
} orc_mixing;

/* Status codes (the reference throws std::runtime_error in these cases). */
enum {
    ORC_OK = 0,
    ORC_BAD_SIZE = 1,        /* empty / mismatched vectors */
    ORC_BAD_ORDER = 2,       /* "radii order messed up" */
    ORC_LAYER_LIMIT = 3,     /* "setMaxlayers : invalid number of maxLayer" */
    ORC_BAD_ARGUMENT = 4
};

/* Earth model after the reference's setDensity (atmoscpupropagator.hpp:116-170):
 * radii sorted descending, per-shell rho / Ye (and a,b,c for the quadratic model). */
typedef struct {
    int n;              /* number of radii rows (including the r=0 row when given) */
    const double* radii;
    const double* rhos; /* constant model (may be NULL when poly) */
    const double* yps;
    const double* as;   /* quadratic model coefficients (NULL when constant) */
    const double* bs;
    const double* cs;
    int poly;           /* 1: density from getDensityOfLayerPoly */
} orc_earth;

/* Sort a user-supplied model into the reference's descending order.  Inputs are the
 * user's vectors (ascending or descending); outputs must hold n doubles each.
 * Returns ORC_BAD_ORDER if the radii are not monotone. */
int orc_flip_model(int n, const double* radii, const double* c1, const double* c2,
                   const double* c3, const double* c4,
                   double* radii_out, double* c1_out, double* c2_out, double* c3_out,
                   double* c4_out);

/* Number of shells crossed for each cosine (setMaxlayers, atmoscpupropagator.hpp:431-444).
 * radii must already be descending. Returns ORC_LAYER_LIMIT when a count exceeds limit. */
int orc_max_layers(const double* radii, int n_radii, const double* cosines, int nc,
                   int limit, int* maxlayers);

/* Atmospheric probabilities, reference CPU layout out[ic][ie][9] (channel a*3+b = P(a->b)).
 * Production-height averaging follows physics.hpp:997-1067; pass avg=0 for the
 * reference's reachable fixed-height path. ph_prob is [2][3][ne][nc][n_ph_bins],
 * ph_edges has n_ph_bins+1 entries in km. */
int orc_atmos(const orc_mixing* mix, int antineutrino,
              const double* cosines, int nc, const double* energies, int ne,
              const orc_earth* earth, double prod_height_km,
              int avg, int n_ph_bins, const double* ph_prob, const double* ph_edges,
              int layer_limit, int nthreads, double* out);

/* Beam probabilities, reference CPU layout out[ie][9] (calculate_beam, physics.hpp:1153-1260). */
int orc_beam(const orc_mixing* mix, int antineutrino, const double* energies, int ne,
             double rho, double path_km, int nthreads, double* out);

/* Single-layer transition amplitude A (row = final flavour, col = initial flavour),
 * interleaved re/im, via getMfast + getA (get_transition_matrix, physics.hpp:603-611). */
void orc_transition_matrix(const orc_mixing* mix, int antineutrino, double E, double rho_e,
                           double L_km, double* A18);

/* Per-cosine trajectory geometry (physics.hpp:745-787, 837, 897-898): segment lengths in
 * km for iLayer = 0..M and the electron densities rho*Ye of each segment.
 * seg_len and seg_rho need room for limit+1 entries. Returns M. */
int orc_trajectory(const orc_earth* earth, double cosine, double prod_height_km, int M,
                   double* seg_len_km, double* seg_rho);

#ifdef __cplusplus
}
#endif
#endif

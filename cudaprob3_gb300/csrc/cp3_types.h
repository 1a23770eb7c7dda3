// cp3_types.h -- plain-old-data blocks shared by the host layer and the kernels.
#pragma once

#include <cstdint>

namespace cp3 {

// Constants of the reference (constants.hpp:26-50, physics.hpp:443): same values.
constexpr double kTwoRtTwoGf = 1.52588e-4;   // 2*sqrt(2)*G_F in the reference's units
constexpr double kKm2Cm = 1.0e5;
constexpr double kREarthKm = 6371.0;
constexpr double kREarthCm = kREarthKm * kKm2Cm;
constexpr double kDensityConvert = 0.5;       // beam Z/A
constexpr double kLoEFac = 2.534;             // (1/2)(1/(hbar c)) in GeV/(eV^2 km)
constexpr int kMaxProdHeightBins = 20;
constexpr int kMaxShells = 128;               // CP3_MAX_SHELLS
constexpr int kMaxSegments = kMaxShells + 1;  // air segment + crossed shells

// One oscillation-parameter set for one neutrino type, as the kernels read it.
// Built on the host from the user's angles and splittings (cp3_host.cpp).
struct alignas(16) OscParams {
    // Reference-faithful data (FP64 kernels): Propagator::Mix_U, DM, mass order.  (The
    // reference's AXFAC bilinears of U serve only its getA, which the rotated-basis beam
    // kernels replace.)
    double U[18];        // U(i,j) re/im at [(i*3+j)*2 + {0,1}]
    double dm[9];        // DM(i,j) = m_i^2 - m_j^2 with the degeneracy break
    // Rotated real basis of the mixed kernels: U = W . O . diag(1,1,e^{-i d}) with
    // W = R23 . diag(1,1,e^{i d}) and O = R13 . R12 real, so 2E.H = W (H0 + V e0 e0^T) W^+.
    double h0[6];        // H0 = O . diag(DM(k,0)) . O^T : 00,01,02,11,12,22 (eV^2)
    double w[4];         // c23, s23, cos d, sin d (d = the dcp actually used in U)
    // det(l - H0 - V e0 e0^T) = l^3 - (t + V) l^2 + (c + V m) l - (D + V n):
    // cpoly = {t = tr H0, c = sum of principal 2x2 minors, D = det H0,
    //          m = h11 + h22, n = h11 h22 - h12^2}
    double cpoly[5];
    // For the mixed kernels' eigen-solver: cpoly as float pairs (hi, lo), and the vacuum
    // eigen-system H0 = O diag(mu) O^T, mu_k = DM(k,0) as float pairs, O in FP32.
    float cpolyf[5][2];
    float muf[3][2];
    float of[3][3];      // O[i][j]; column j is the vacuum eigenvector of mu_j
    float oflo[3][3];    // O - of, the low words (double-float O for the eigenvector tables)
    int order[3];        // root order from the vacuum cubic (prepare_getMfast)
    int anti;            // 1: antineutrino sign of the matter potential
    float wf[4];         // w rounded to float (the mixed kernels' W)
};

}  // namespace cp3

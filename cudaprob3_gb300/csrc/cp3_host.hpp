// cp3_host.hpp -- host side of the propagator: parameter blocks, Earth model ingest,
// per-cosine trajectory tables, model-file parsing.  No CUDA in here.
#pragma once

#include <string>
#include <vector>

#include "cp3_types.h"

namespace cp3 {

struct MixingInput {
    double theta12 = 0, theta13 = 0, theta23 = 0, dcp = 0;
    int knutype = 1;
    double dm12sq = 0, dm23sq = 0;
};

// Propagator::setMNSMatrix + setNeutrinoMasses (propagator.hpp:148-209),
// physics::setMixMatrix (physics.hpp:130-152) and prepare_getMfast (:198-252), plus the
// rotated-basis data of the mixed kernels.
void build_osc_params(const MixingInput& m, int antineutrino, OscParams* out);

// Earth model in the reference's internal order: radii descending (first row = surface),
// row i carrying the shell between radii[i+1] and radii[i]
// (AtmosCpuPropagator::setDensity, atmoscpupropagator.hpp:116-170, 181-242).
struct EarthModel {
    std::vector<double> radii, rho, ye, a, b, c;
    bool poly = false;
    std::vector<double> coslimit;  // atmoscpupropagator.hpp:160-167
};

// Validates sizes and order, flips to descending, fills coslimit. Returns a CP3 status.
int make_earth_model(const double* radii, const double* c1, const double* c2,
                     const double* c3, const double* ye, int n, bool poly, EarthModel* out,
                     std::string* err);

// setMaxlayers (atmoscpupropagator.hpp:431-444): shells crossed by cos(zenith).
int count_shells(const EarthModel& e, double cosz);

// One flattened row per cosine: segments l = 0..M (air, then shells inwards), each with
// its length in km, its electron density rho*Ye and its density class (0 = air,
// 1 + i = shell i of the constant model; -1 for the polynomial model).
struct TrajectoryTable {
    std::vector<int> offset;       // n_cosines + 1
    std::vector<double> len_km;    // segments
    std::vector<double> rho_e;     // segments
    std::vector<int> cls;          // segments
    std::vector<int> maxlayers;    // n_cosines
    std::vector<double> air_cm;    // n_cosines: segment 0 in cm, as calculate_atmos's `dist`
    std::vector<double> path_cm;   // n_cosines: PathLength (physics.hpp:897-898)
    int max_segments = 0;
};

// Production-height averaging (physics.hpp:1020-1027): for every cosine the shift of the
// path length at each bin edge, PathLength(edge) - PathLength, cm; out[ic * (nb+1) + p].
void production_height_shifts(const double* cosines, int nc, double height_cm,
                              const double* edges_km, int nb, std::vector<double>* out);

// Geometry of physics::calculate_atmos (physics.hpp:837, 897-898) and
// getTraversedDistanceOfLayer / getDensityOfLayer / getDensityOfLayerPoly (:634-787).
int build_trajectories(const EarthModel& e, const double* cosines, int nc, double height_cm,
                       TrajectoryTable* out, std::string* err);

// Text model file (atmoscpupropagator.hpp:250-344).  2, 3 or 5 numeric columns.
int parse_model_file(const char* path, int* ncols, std::vector<std::vector<double>>* cols,
                     std::string* err);

}  // namespace cp3

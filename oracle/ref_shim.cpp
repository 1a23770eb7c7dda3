// ref_shim.cpp -- extern "C" glue around the reference's own CPU propagators
// (TEST INFRASTRUCTURE ONLY; built by `make -C oracle ref` in a container that has the
// reference sources, output oracle/_ref/libcp3ref.so, never shipped).
//
// The reference headers are compiled where they lie (-I points at the reference tree).
// Only one thing is changed, from outside: the reference's Constants<T> (constants.hpp:24-50)
// caps trajectories at MaxNLayers()==10 crossed shells, which rejects the 12- and 59-shell
// profiles used by the precision study.  This file pre-empts that header through its include
// guard and supplies the same constants with MaxNLayers()==64.
#include <hpc_helpers.cuh>

#define CUDAPROB3_CONSTANTS_HPP
namespace cudaprob3linear {
template <typename FLOAT_T>
struct Constants {
    static constexpr FLOAT_T tworttwoGf() { return 1.52588e-4; }
    static constexpr FLOAT_T km2cm() { return 1.0e5; }
    static constexpr FLOAT_T REarth() { return 6371.0; }
    static constexpr FLOAT_T REarthcm() { return REarth() * km2cm(); }
    static constexpr FLOAT_T density_convert() { return 0.5; }
    static constexpr int MaxProdHeightBins() { return 20; }
    static constexpr int MaxNLayers() { return 64; }
    static constexpr FLOAT_T Epsilon() { return 1e-6; }
};
}  // namespace cudaprob3linear

#include <atmoscpupropagator.hpp>
#include <beamcpupropagator.hpp>

#include <chrono>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

using namespace cudaprob3linear;

namespace {
std::string g_last_error;

// Gives the shim access to the propagator's protected state so the production-height
// averaging branch of physics::calculate_atmos can be driven directly (the public
// SetNumberOfProductionHeightBinsForAveraging never enables it,
// atmoscpupropagator.hpp:97-99).
struct AtmosProbe : public AtmosCpuPropagator<double> {
    AtmosProbe(int nc, int ne, int nt) : AtmosCpuPropagator<double>(nc, ne, nt) {}
    void run_averaged(NeutrinoType type, int nbins, const double* prob, const double* edges,
                      double* out) {
        std::vector<double> p(size_t(Constants<double>::MaxProdHeightBins()) * 2 * 3 *
                                  this->n_energies * this->n_cosines,
                              0.0);
        std::memcpy(p.data(), prob, sizeof(double) * size_t(nbins) * 2 * 3 * this->n_energies *
                                        this->n_cosines);
        std::vector<double> e(Constants<double>::MaxProdHeightBins() + 1, 0.0);
        std::memcpy(e.data(), edges, sizeof(double) * size_t(nbins + 1));
        physics::setMixMatrix_host(this->Mix_U.data());
        physics::setMassDifferences_host(this->dm.data());
        physics::calculate_atmos(type, this->cosineList.data(), this->cosineList.size(),
                                 this->energyList.data(), this->energyList.size(),
                                 this->radii.data(), this->as.data(), this->bs.data(),
                                 this->cs.data(), this->rhos.data(), this->yps.data(),
                                 this->maxlayers.data(), this->ProductionHeightinCentimeter, true,
                                 nbins, p.data(), e.data(), this->UsePolyDensity, out);
    }
};

std::vector<double> vec(const double* p, int n) { return std::vector<double>(p, p + n); }
}  // namespace

extern "C" {

const char* ref_last_error() { return g_last_error.c_str(); }

// One full atmospheric computation through the reference's public API
// (example/mainatmos.cpp:111-147 call order).  out: [nc][ne][9].
// poly=0: c1 = rho.  poly=1: c1,c2,c3 = a,b,c.  avg>0: production-height averaging.
// reps>0 times calculateProbabilities (median-free: returns total seconds in *secs).
int ref_atmos(double t12, double t13, double t23, double dcp, int knutype, double dm12,
              double dm23, int antineutrino, const double* cosines, int nc,
              const double* energies, int ne, const double* radii, const double* c1,
              const double* c2, const double* c3, const double* yps, int nr, int poly,
              double h_km, int avg_bins, const double* ph_prob, const double* ph_edges,
              int nthreads, int reps, double* secs, double* out) {
    try {
        AtmosProbe p(nc, ne, nthreads > 0 ? nthreads : 1);
        p.setEnergyList(vec(energies, ne));
        p.setCosineList(vec(cosines, nc));
        p.setMNSMatrix(t12, t13, t23, dcp, knutype);
        p.setNeutrinoMasses(dm12, dm23);
        if (poly)
            p.setDensity(vec(radii, nr), vec(c1, nr), vec(c2, nr), vec(c3, nr), vec(yps, nr));
        else
            p.setDensity(vec(radii, nr), vec(c1, nr), vec(yps, nr));
        p.setProductionHeight(h_km);
        const NeutrinoType t = antineutrino ? Antineutrino : Neutrino;
        if (avg_bins > 0) {
            p.run_averaged(t, avg_bins, ph_prob, ph_edges, out);
            return 0;
        }
        const int n = reps > 0 ? reps : 1;
        auto t0 = std::chrono::steady_clock::now();
        for (int r = 0; r < n; r++) p.calculateProbabilities(t);
        auto t1 = std::chrono::steady_clock::now();
        if (secs) *secs = std::chrono::duration<double>(t1 - t0).count();
        for (int ic = 0; ic < nc; ic++)
            for (int ie = 0; ie < ne; ie++)
                for (int c = 0; c < 9; c++)
                    out[(size_t(ic) * ne + ie) * 9 + c] = p.getProbability(ic, ie, ProbType(c));
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

// Beam through the reference's public API (example/mainbeam.cpp:107-131).  out: [ne][9].
int ref_beam(double t12, double t13, double t23, double dcp, int knutype, double dm12,
             double dm23, int antineutrino, const double* energies, int ne, double rho,
             double L_km, int nthreads, int reps, double* secs, double* out) {
    try {
        BeamCpuPropagator<double> p(ne, nthreads > 0 ? nthreads : 1);
        p.setEnergyList(vec(energies, ne));
        p.setMNSMatrix(t12, t13, t23, dcp, knutype);
        p.setNeutrinoMasses(dm12, dm23);
        p.setDensity(rho);
        p.setPathLength(L_km);
        const NeutrinoType t = antineutrino ? Antineutrino : Neutrino;
        const int n = reps > 0 ? reps : 1;
        auto t0 = std::chrono::steady_clock::now();
        for (int r = 0; r < n; r++) p.calculateProbabilities(t);
        auto t1 = std::chrono::steady_clock::now();
        if (secs) *secs = std::chrono::duration<double>(t1 - t0).count();
        for (int ie = 0; ie < ne; ie++)
            for (int c = 0; c < 9; c++) out[size_t(ie) * 9 + c] = p.getProbability(ie, ProbType(c));
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

}  // extern "C"

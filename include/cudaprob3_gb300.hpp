// cudaprob3_gb300.hpp -- C++ facade with the reference's class names and signatures.
//
// Header-only, over the C ABI of libcp3gb300.so (cudaprob3_gb300.h).  Code written against
// CUDAProb3++'s AtmosCudaPropagatorSingle / BeamCudaPropagatorSingle (namespace
// cudaprob3linear) compiles against this header unchanged; link with -lcp3gb300.  Non-zero
// ABI statuses become std::runtime_error carrying the reference's message; nothing calls
// exit().
#pragma once

#include <cstddef>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "cudaprob3_gb300.h"

namespace cudaprob3linear {

// types.hpp:23-29
enum ProbType : int { e_e = 0, e_m = 1, e_t = 2, m_e = 3, m_m = 4, m_t = 5, t_e = 6, t_m = 7, t_t = 8 };
enum NeutrinoType { Neutrino, Antineutrino };

// Constants<FLOAT_T> (constants.hpp:24-50): same values; the crossed-shell limit is the
// runtime CP3_MAX_SHELLS instead of the reference's compile-time 10.
template <typename FLOAT_T>
struct Constants {
    static constexpr FLOAT_T tworttwoGf() { return 1.52588e-4; }
    static constexpr FLOAT_T km2cm() { return 1.0e5; }
    static constexpr FLOAT_T REarth() { return 6371.0; }
    static constexpr FLOAT_T REarthcm() { return REarth() * km2cm(); }
    static constexpr FLOAT_T density_convert() { return 0.5; }
    static constexpr int MaxProdHeightBins() { return 20; }
    static constexpr int MaxNLayers() { return CP3_MAX_SHELLS; }
    static constexpr FLOAT_T Epsilon() { return 1e-6; }
};

namespace detail {
inline void check(int rc, const cp3_propagator* h) {
    if (rc != CP3_OK) throw std::runtime_error(cp3_last_error(h));
}
}  // namespace detail

// Propagator<FLOAT_T> (propagator.hpp:45-300).  The handle owns every buffer; copying is
// disabled (the reference's GPU classes delete their copy constructors too).
template <class FLOAT_T>
class Propagator {
public:
    Propagator(const Propagator&) = delete;
    Propagator& operator=(const Propagator&) = delete;
    Propagator(Propagator&& o) noexcept : h_(o.h_), n_cosines(o.n_cosines), n_energies(o.n_energies) { o.h_ = nullptr; }
    virtual ~Propagator() { cp3_destroy(h_); }

    virtual void setMNSMatrix(FLOAT_T theta12, FLOAT_T theta13, FLOAT_T theta23, FLOAT_T dCP,
                              int kNuType) {
        detail::check(cp3_set_mns(h_, theta12, theta13, theta23, dCP, kNuType), h_);
    }
    virtual void setNeutrinoMasses(FLOAT_T dm12sq, FLOAT_T dm23sq) {
        detail::check(cp3_set_masses(h_, dm12sq, dm23sq), h_);
    }
    virtual void setEnergyList(const std::vector<FLOAT_T>& list) {
        const std::vector<double> d(list.begin(), list.end());
        detail::check(cp3_set_energies(h_, d.data(), (int)d.size()), h_);
    }
    virtual void setChemicalComposition(const std::vector<FLOAT_T>& list) = 0;
    virtual void calculateProbabilities(NeutrinoType type) {
        detail::check(cp3_calculate(h_, type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO), h_);
    }
    virtual void getProbabilityArr(FLOAT_T* probArr, ProbType t) {
        std::vector<double> tmp((size_t)n_energies * (n_cosines > 0 ? n_cosines : 1));
        detail::check(cp3_get_probability_arr(h_, (int)t, tmp.data()), h_);
        for (size_t i = 0; i < tmp.size(); i++) probArr[i] = (FLOAT_T)tmp[i];
    }
    virtual void setPathLength(FLOAT_T path_length) = 0;
    virtual void setDensity(FLOAT_T rho) = 0;

    // Additions (no reference counterpart).
    void calculateProbabilitiesAsync(NeutrinoType type, void* cuda_stream = nullptr) {
        detail::check(cp3_calculate_async(h_, type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO,
                                          cuda_stream), h_);
    }
    // Compute and copy the result (device layout) to page-locked host memory, pipelined.
    void calculateProbabilitiesToHostAsync(NeutrinoType type, void* host_dst, int n_chunks = 0,
                                           void* cuda_stream = nullptr) {
        detail::check(cp3_calculate_to_host_async(
                          h_, type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO, host_dst,
                          n_chunks, cuda_stream), h_);
    }
    void waitForCompletion() { detail::check(cp3_synchronize(h_), h_); }
    cp3_propagator* handle() { return h_; }

protected:
    Propagator() = default;
    cp3_propagator* h_ = nullptr;
    int n_cosines = 0;
    int n_energies = 0;
};

// AtmosCudaPropagatorSingle (atmoscudapropagator.cuh:41-132).  `precision` is an addition:
// CP3_FP64 (default, the drop-in) or CP3_MIXED.
class AtmosCudaPropagatorSingle : public Propagator<double> {
public:
    AtmosCudaPropagatorSingle(int id, int n_cosines_, int n_energies_, int precision = CP3_FP64) {
        detail::check(cp3_atmos_create(id, n_cosines_, n_energies_, precision, &h_), nullptr);
        n_cosines = n_cosines_;
        n_energies = n_energies_;
    }
    AtmosCudaPropagatorSingle(int n_cosines_, int n_energies_)
        : AtmosCudaPropagatorSingle(0, n_cosines_, n_energies_) {}

    void setCosineList(const std::vector<double>& list) {
        detail::check(cp3_set_cosines(h_, list.data(), (int)list.size()), h_);
    }
    void setDensity(const std::vector<double>& radii_, const std::vector<double>& rhos_,
                    const std::vector<double>& yps_) {
        if (rhos_.size() != radii_.size()) throw std::runtime_error("setDensity : rhos.size() != radii.size()");
        if (rhos_.size() != yps_.size()) throw std::runtime_error("setDensity : rhos.size() != yps.size()");
        detail::check(cp3_set_layers(h_, radii_.data(), rhos_.data(), yps_.data(), (int)radii_.size()), h_);
    }
    void setDensity(const std::vector<double>& radii_, const std::vector<double>& a_,
                    const std::vector<double>& b_, const std::vector<double>& c_,
                    const std::vector<double>& yps_) {
        if (a_.size() != radii_.size()) throw std::runtime_error("setDensity : a.size() != radii.size()");
        if (a_.size() != yps_.size()) throw std::runtime_error("setDensity : a.size() != yps.size()");
        if (b_.size() != a_.size() || c_.size() != a_.size())
            throw std::runtime_error("setDensity : vectors must not be empty");
        detail::check(cp3_set_layers_poly(h_, radii_.data(), a_.data(), b_.data(), c_.data(),
                                          yps_.data(), (int)radii_.size()), h_);
    }
    // atmoscpupropagator.hpp:347-358: a printing dummy in the reference.
    void setDensity(double) override {
        std::fprintf(stderr, "DUMMY FUNCTION: ATMOS class uses setDensity(radii, rhos, yps), "
                             "setDensity(radii, a, b, c, yps) or setDensityFromFile(filename)\n");
    }
    void setDensityFromFile(const std::string& filename, double ye_core = 0.468,
                            double ye_mantle = 0.497) {
        detail::check(cp3_set_density_file(h_, filename.c_str(), ye_core, ye_mantle), h_);
    }
    void setChemicalComposition(const std::vector<double>& list) override {
        detail::check(cp3_set_chemical_composition(h_, list.data(), (int)list.size()), h_);
    }
    // AtmosCpuPropagator::getNlayerBoundaries (atmoscpupropagator.hpp:85): the density
    // model's rows (layers + 1), after any density setter.
    virtual int getNlayerBoundaries() {
        int n = 0;
        detail::check(cp3_get_n_layer_boundaries(h_, &n), h_);
        return n;
    }
    void setProductionHeight(double heightKM) {
        detail::check(cp3_set_production_height(h_, heightKM), h_);
    }
    void setPathLength(double) override {
        std::fprintf(stderr, "DUMMY FUNCTION - ATMOS class calculates PATH LENGTH\n");
    }
    // SetNumberOfProductionHeightBinsForAveraging + setProductionHeightList
    // (atmoscpupropagator.hpp:85-110, 395-427); n >= 1 enables averaging here.
    void SetNumberOfProductionHeightBinsForAveraging(int n) {
        if (n < 0 || n > 20)
            throw std::runtime_error("SetNumberOfProductionHeightBinsForAveraging : invalid number of production height bins");
        avg_bins_ = n;
        if (n == 0) detail::check(cp3_set_production_height_averaging(h_, 0, nullptr, nullptr), h_);
    }
    void setProductionHeightList(const std::vector<double>& list_prob, const std::vector<double>& list_bins) {
        if (avg_bins_ < 1)
            throw std::runtime_error("Propagator::setProductionHeightList. Trying to set Production Height information but propagator is not expecting to use it");
        if (list_prob.size() != (size_t)avg_bins_ * 2 * 3 * n_energies * n_cosines)
            throw std::runtime_error("Propagator::setProductionHeightList. Prob array is not the expected size");
        if (list_bins.size() != (size_t)avg_bins_ + 1)
            throw std::runtime_error("Propagator::setProductionHeightList. ProductionHeightBins array is not expected size");
        detail::check(cp3_set_production_height_averaging(h_, avg_bins_, list_prob.data(), list_bins.data()), h_);
    }
    double getProbability(int index_cosine, int index_energy, ProbType t) {
        double v = 0;
        detail::check(cp3_get_probability(h_, index_cosine, index_energy, (int)t, &v), h_);
        return v;
    }

private:
    int avg_bins_ = 0;
};

// BeamCudaPropagatorSingle (beamcudapropagator.cuh:41-120).
class BeamCudaPropagatorSingle : public Propagator<double> {
public:
    // The reference's two constructors (beamcudapropagator.cuh:52,57): (id, n_energies,
    // n_threads) and (n_energies, n_threads), so a two-argument call means what it means
    // there.  n_threads is the OpenMP thread count of the reference's CPU base class.
    BeamCudaPropagatorSingle(int id, int n_energies_, int n_threads, int precision = CP3_FP64) {
        (void)n_threads;
        detail::check(cp3_beam_create(id, n_energies_, precision, &h_), nullptr);
        n_energies = n_energies_;
    }
    BeamCudaPropagatorSingle(int n_energies_, int n_threads)
        : BeamCudaPropagatorSingle(0, n_energies_, n_threads) {}
    void setDensity(double rho) override { detail::check(cp3_set_beam_density(h_, rho), h_); }
    void setPathLength(double path_length) override {
        detail::check(cp3_set_beam_path_length(h_, path_length), h_);
    }
    void setChemicalComposition(const std::vector<double>&) override {
        throw std::runtime_error("BeamCpuPropagator::setChemicalComposition. Size of input list not equal to expectation");
    }
    double getProbability(int index_energy, ProbType t) {
        double v = 0;
        detail::check(cp3_get_probability_beam(h_, index_energy, (int)t, &v), h_);
        return v;
    }
};

// The legacy template name (cudapropagator.cuh:40): FLOAT_T = double selects the FP64
// kernels, FLOAT_T = float the mixed-precision kernels.  Results are read as double.
template <class FLOAT_T>
class CudaPropagatorSingle : public AtmosCudaPropagatorSingle {
public:
    CudaPropagatorSingle(int id, int n_cosines_, int n_energies_)
        : AtmosCudaPropagatorSingle(id, n_cosines_, n_energies_,
                                    sizeof(FLOAT_T) == sizeof(double) ? CP3_FP64 : CP3_MIXED) {}
    CudaPropagatorSingle(int n_cosines_, int n_energies_) : CudaPropagatorSingle(0, n_cosines_, n_energies_) {}
};

// ---- additions with no reference counterpart: batches and the serving loop --------------

// Many problems (own grids, own parameters) in one run of a persistent kernel (cp3_batch_*).
class PropagatorBatch {
public:
    explicit PropagatorBatch(int device = 0) { check(cp3_batch_create(device, &b_)); }
    ~PropagatorBatch() { cp3_batch_destroy(b_); }
    PropagatorBatch(const PropagatorBatch&) = delete;
    PropagatorBatch& operator=(const PropagatorBatch&) = delete;

    void setEarth(const std::vector<double>& radii, const std::vector<double>& rho,
                  const std::vector<double>& ye, double production_height_km) {
        if (rho.size() != radii.size() || ye.size() != radii.size())
            throw std::runtime_error("PropagatorBatch::setEarth. radii, rho and ye differ in size");
        check(cp3_batch_set_earth(b_, radii.data(), rho.data(), ye.data(), (int)radii.size(),
                                  production_height_km));
    }
    int addAtmospheric(const std::vector<double>& cosines, const std::vector<double>& energies) {
        int id = -1;
        check(cp3_batch_add_atmos(b_, cosines.data(), (int)cosines.size(), energies.data(),
                                  (int)energies.size(), &id));
        return id;
    }
    int addBeam(const std::vector<double>& energies, double rho,
                const std::vector<double>& baselines_km) {
        int id = -1;
        check(cp3_batch_add_beam(b_, energies.data(), (int)energies.size(), rho,
                                 baselines_km.data(), (int)baselines_km.size(), &id));
        return id;
    }
    // setMNSMatrix + setNeutrinoMasses + the neutrino type of one problem.
    void setParameters(int id, double theta12, double theta13, double theta23, double dcp,
                       int kNuType, double dm12sq, double dm23sq, NeutrinoType type) {
        check(cp3_batch_set_params(b_, id, theta12, theta13, theta23, dcp, kNuType, dm12sq,
                                   dm23sq, type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO));
    }
    void commit() { check(cp3_batch_commit(b_)); }
    void tune(bool use_cache = true) { check(cp3_batch_tune(b_, use_cache ? 1 : 0)); }
    void run(void* cuda_stream = nullptr) { check(cp3_batch_run(b_, cuda_stream)); }
    // One run with every result copied to dst (result bytes, laid out as the arena), the
    // download of each window of problems overlapping the next window's computation.
    void runToHost(void* dst, int n_pieces = 0, void* cuda_stream = nullptr) {
        check(cp3_batch_run_to_host(b_, dst, n_pieces, cuda_stream));
    }
    double synchronize() {
        double ms = 0.0;
        check(cp3_batch_synchronize(b_, &ms));
        return ms;
    }
    // Device result of one problem: atmospheric [9][n_cosines][n_energies], beam
    // [n_baselines][9][n_energies] floats.
    const float* deviceResult(int id, size_t* count = nullptr) {
        const float* p = nullptr;
        check(cp3_batch_result(b_, id, &p, count));
        return p;
    }
    std::vector<float> result(int id) {
        size_t n = 0;
        deviceResult(id, &n);
        std::vector<float> out(n);
        check(cp3_batch_copy_result(b_, id, out.data(), nullptr));
        synchronizeCopies();
        return out;
    }
    // Float offset of problem id's result in the result arena, and an asynchronous copy of
    // the arena's floats [first, first + count) (on the batch's stream when stream is null).
    size_t resultOffset(int id) {
        size_t off = 0;
        check(cp3_batch_result_offset(b_, id, &off));
        return off;
    }
    void copyResultsAsync(size_t first, size_t count, void* dst, void* stream = nullptr) {
        check(cp3_batch_copy_results(b_, first, count, dst, stream));
    }
    cp3_batch* handle() { return b_; }

private:
    void check(int rc) {
        if (rc != CP3_OK) throw std::runtime_error(cp3_batch_last_error(b_));
    }
    void synchronizeCopies() { check(cp3_batch_synchronize(b_, nullptr)); }  // the batch stream too
    cp3_batch* b_ = nullptr;
};

// Continuous batching for many concurrent callers (cp3_server_*).
class PropagatorServer {
public:
    PropagatorServer(int device, size_t pool_bytes, int max_batch = 256,
                     long long max_bins_per_launch = 8000000) {
        check(cp3_server_create(device, pool_bytes, max_batch, max_bins_per_launch, &s_));
    }
    ~PropagatorServer() { cp3_server_destroy(s_); }
    PropagatorServer(const PropagatorServer&) = delete;
    PropagatorServer& operator=(const PropagatorServer&) = delete;

    void setEarth(const std::vector<double>& radii, const std::vector<double>& rho,
                  const std::vector<double>& ye, double production_height_km) {
        if (rho.size() != radii.size() || ye.size() != radii.size())
            throw std::runtime_error("PropagatorServer::setEarth. radii, rho and ye differ in size");
        check(cp3_server_set_earth(s_, radii.data(), rho.data(), ye.data(), (int)radii.size(),
                                   production_height_km));
    }
    int addAtmosphericGrid(const std::vector<double>& cosines, const std::vector<double>& energies) {
        int g = -1;
        check(cp3_server_add_atmos_grid(s_, cosines.data(), (int)cosines.size(), energies.data(),
                                        (int)energies.size(), &g));
        return g;
    }
    int addBeamGrid(const std::vector<double>& energies, double rho,
                    const std::vector<double>& baselines_km) {
        int g = -1;
        check(cp3_server_add_beam_grid(s_, energies.data(), (int)energies.size(), rho,
                                       baselines_km.data(), (int)baselines_km.size(), &g));
        return g;
    }
    void start() { check(cp3_server_start(s_)); }
    unsigned long long submit(int grid, double theta12, double theta13, double theta23,
                              double dcp, int kNuType, double dm12sq, double dm23sq,
                              NeutrinoType type) {
        unsigned long long id = 0;
        check(cp3_server_submit(s_, grid, theta12, theta13, theta23, dcp, kNuType, dm12sq, dm23sq,
                                type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO, &id));
        return id;
    }
    bool wait(unsigned long long id, double timeout_s) {
        int done = 0;
        check(cp3_server_wait(s_, id, timeout_s, &done));
        return done != 0;
    }
    std::vector<float> result(unsigned long long id, double* latency_ms = nullptr) {
        const float* p = nullptr;
        size_t n = 0;
        check(cp3_server_result(s_, id, &p, &n, latency_ms));
        std::vector<float> out(n);
        check(cp3_server_copy_result(s_, id, out.data()));
        return out;
    }
    void release(unsigned long long id) { check(cp3_server_release(s_, id)); }
    // Ids finished since the previous poll, in completion order (waits up to timeout_s while
    // there is none); call poll(0, 0.0) once before the first submit to start recording.
    std::vector<unsigned long long> poll(int max_ids, double timeout_s) {
        std::vector<unsigned long long> ids((size_t)(max_ids > 0 ? max_ids : 0));
        int n = 0;
        check(cp3_server_poll(s_, ids.data(), max_ids, timeout_s, &n));
        ids.resize((size_t)n);
        return ids;
    }
    cp3_server* handle() { return s_; }

private:
    void check(int rc) {
        if (rc != CP3_OK) throw std::runtime_error(cp3_server_last_error(s_));
    }
    cp3_server* s_ = nullptr;
};

}  // namespace cudaprob3linear

// ref_gpu_main.cu -- timing driver for the reference's own FP64 CUDA propagators
// (TEST AND BENCH INFRASTRUCTURE ONLY; built by `make -C oracle refgpu REF=<reference tree>`,
// output oracle/_ref/refgpu_bench, never shipped or linked by the product).
//
// It compiles the reference's AtmosCudaPropagatorSingle / BeamCudaPropagatorSingle
// (atmoscudapropagator.cu, beamcudapropagator.cu) where they lie and runs them through their
// public API in the call order of example/mainatmos.cpp:111-147 and example/mainbeam.cpp:107-131.
// Only one thing is changed, from outside: Constants<T>::MaxNLayers() (constants.hpp:46) is
// raised from 10 to 64 through the header's include guard, as in ref_shim.cpp, so that the
// 59-shell precision-study Earth is accepted.
//
// The reference reports CUDA errors by printing and calling exit(1) (hpc_helpers.cuh:71-78),
// so bench.py runs this program as a child process: a failure ends the child, not the bench.
//
// Usage: refgpu_bench <input.txt> <sample_out.bin>
//   input.txt (whitespace separated):
//     kind atmos|beam   steps K   warmup W
//     params t12 t13 t23 dcp dm12sq dm23sq
//     atmos: height_km h   cosines n c_0..c_{n-1}   model n (r rho ye)x n   sample_every s
//     beam:  rho g/cm3     length_km L
//     energies n e_0..e_{n-1}
//   stdout: one JSON object {"ms_per_call": [[nu, nubar] per step], ...}
//   sample_out.bin: float64 probabilities of every s-th cosine row (atmos) or of every
//     energy (beam), [type][row][energy][9], channel a*3+b = P(a->b), read through
//     getProbability (the reference's own result path).
//
// kind batch: many problems, as a caller without batching runs them -- one propagator per
// problem (created before the timed region), calculateProbabilities on each in turn:
//     kind batch   steps K   warmup W   sample_every s   height_km h   model n (r rho ye)x n
//     problem atmos t12 t13 t23 dcp dm12sq dm23sq anti   cosines n ...   energies n ...
//     problem beam  t12 t13 t23 dcp dm12sq dm23sq anti   rho r   length_km L   energies n ...
//   stdout: {"ms_per_step": [total over the problems, per step], ...}
//   sample_out.bin: per problem in order, every s-th cosine row (atmos: [row][energy][9]) or
//     every s-th energy (beam: [energy][9]).
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

#include <hpc_helpers.cuh>
#include <atmoscudapropagator.cu>
#include <beamcudapropagator.cu>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace cudaprob3linear;

namespace {

struct Problem {
    bool atmos = true;
    double t12 = 0, t13 = 0, t23 = 0, dcp = 0, dm12 = 0, dm23 = 0;
    int anti = 0;
    double rho = 0, length = 0;
    std::vector<double> cosines, energies;
};

struct Input {
    std::string kind;
    std::vector<Problem> problems;
    int steps = 5, warmup = 1, sample_every = 1;
    double t12 = 0, t13 = 0, t23 = 0, dcp = 0, dm12 = 0, dm23 = 0;
    double height = 0, rho = 0, length = 0;
    std::vector<double> cosines, energies, radii, rhos, yes;
};

std::vector<double> read_list(std::istream& in) {
    int n = 0;
    in >> n;
    if (!in || n < 0) throw std::runtime_error("bad list length");
    std::vector<double> v(n);
    for (double& x : v) in >> x;
    if (!in) throw std::runtime_error("short list");
    return v;
}

Input read_input(const char* path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error(std::string("cannot open ") + path);
    Input p;
    std::string key;
    while (in >> key) {
        if (key == "kind") in >> p.kind;
        else if (key == "steps") in >> p.steps;
        else if (key == "warmup") in >> p.warmup;
        else if (key == "params") in >> p.t12 >> p.t13 >> p.t23 >> p.dcp >> p.dm12 >> p.dm23;
        else if (key == "height_km") in >> p.height;
        else if (key == "rho") in >> p.rho;
        else if (key == "length_km") in >> p.length;
        else if (key == "sample_every") in >> p.sample_every;
        else if (key == "cosines") p.cosines = read_list(in);
        else if (key == "energies") p.energies = read_list(in);
        else if (key == "problem") {
            Problem q;
            std::string k;
            in >> k >> q.t12 >> q.t13 >> q.t23 >> q.dcp >> q.dm12 >> q.dm23 >> q.anti;
            q.atmos = k == "atmos";
            if (!q.atmos && k != "beam") throw std::runtime_error("problem kind must be atmos or beam");
            std::string sub;
            if (q.atmos) {
                in >> sub;
                if (sub != "cosines") throw std::runtime_error("atmos problem: cosines expected");
                q.cosines = read_list(in);
            } else {
                in >> sub >> q.rho;
                if (sub != "rho") throw std::runtime_error("beam problem: rho expected");
                in >> sub >> q.length;
                if (sub != "length_km") throw std::runtime_error("beam problem: length_km expected");
            }
            in >> sub;
            if (sub != "energies") throw std::runtime_error("problem: energies expected");
            q.energies = read_list(in);
            p.problems.push_back(q);
        }
        else if (key == "model") {
            int n = 0;
            in >> n;
            for (int i = 0; i < n; i++) {
                double r, d, y;
                in >> r >> d >> y;
                p.radii.push_back(r);
                p.rhos.push_back(d);
                p.yes.push_back(y);
            }
        } else throw std::runtime_error("unknown key " + key);
        if (!in) throw std::runtime_error("malformed value after " + key);
    }
    if (p.energies.empty() && p.problems.empty()) throw std::runtime_error("no energies");
    if (p.sample_every < 1) p.sample_every = 1;
    return p;
}

template <class P>
double call_ms(P& prop, NeutrinoType t) {
    const auto a = std::chrono::steady_clock::now();
    prop.calculateProbabilities(t);  // launch + cudaStreamSynchronize in the reference
    const auto b = std::chrono::steady_clock::now();
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// The batch form: one propagator per problem, each computed in turn through the reference's
// synchronous calculateProbabilities.
int run_batch(const Input& p, const char* sample_path) {
    std::vector<std::unique_ptr<AtmosCudaPropagatorSingle>> atm;
    std::vector<std::unique_ptr<BeamCudaPropagatorSingle>> beam;
    std::vector<std::pair<bool, size_t>> order;  // (atmos?, index) per problem
    long long bins = 0;
    for (const Problem& q : p.problems) {
        const int ne = (int)q.energies.size();
        if (q.atmos) {
            const int nc = (int)q.cosines.size();
            atm.emplace_back(new AtmosCudaPropagatorSingle(0, nc, ne));
            AtmosCudaPropagatorSingle& a = *atm.back();
            a.setEnergyList(q.energies);
            a.setCosineList(q.cosines);
            a.setMNSMatrix(q.t12, q.t13, q.t23, q.dcp, q.anti ? -1 : 1);
            a.setNeutrinoMasses(q.dm12, q.dm23);
            a.setDensity(p.radii, p.rhos, p.yes);
            a.setProductionHeight(p.height);
            order.emplace_back(true, atm.size() - 1);
            bins += (long long)nc * ne;
        } else {
            beam.emplace_back(new BeamCudaPropagatorSingle(0, ne, 1));
            BeamCudaPropagatorSingle& b = *beam.back();
            b.setEnergyList(q.energies);
            b.setMNSMatrix(q.t12, q.t13, q.t23, q.dcp, q.anti ? -1 : 1);
            b.setNeutrinoMasses(q.dm12, q.dm23);
            b.setDensity(q.rho);
            b.setPathLength(q.length);
            order.emplace_back(false, beam.size() - 1);
            bins += ne;
        }
    }
    auto step = [&]() {
        double total = 0.0;
        for (size_t i = 0; i < order.size(); i++) {
            const NeutrinoType t = p.problems[i].anti ? Antineutrino : Neutrino;
            total += order[i].first ? call_ms(*atm[order[i].second], t) : call_ms(*beam[order[i].second], t);
        }
        return total;
    };
    for (int w = 0; w < p.warmup; w++) step();
    std::vector<double> ms;
    for (int s = 0; s < p.steps; s++) ms.push_back(step());
    std::vector<double> sample;
    for (size_t i = 0; i < order.size(); i++) {
        const Problem& q = p.problems[i];
        const int ne = (int)q.energies.size();
        if (order[i].first) {
            AtmosCudaPropagatorSingle& a = *atm[order[i].second];
            for (int ic = 0; ic < (int)q.cosines.size(); ic += p.sample_every)
                for (int ie = 0; ie < ne; ie++)
                    for (int c = 0; c < 9; c++) sample.push_back(a.getProbability(ic, ie, ProbType(c)));
        } else {
            BeamCudaPropagatorSingle& b = *beam[order[i].second];
            for (int ie = 0; ie < ne; ie += p.sample_every)
                for (int c = 0; c < 9; c++) sample.push_back(b.getProbability(ie, ProbType(c)));
        }
    }
    FILE* f = std::fopen(sample_path, "wb");
    if (!f) throw std::runtime_error("cannot write the sample file");
    const size_t wrote = std::fwrite(sample.data(), sizeof(double), sample.size(), f);
    std::fclose(f);
    if (wrote != sample.size()) throw std::runtime_error("short write of the sample file");
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, 0);
    std::printf("{\"kind\": \"batch\", \"device\": \"%s\", \"problems\": %d, \"bins\": %lld, "
                "\"sample_every\": %d, \"ms_per_step\": [",
                prop.name, (int)order.size(), bins, p.sample_every);
    for (size_t s = 0; s < ms.size(); s++) std::printf("%s%.6f", s ? ", " : "", ms[s]);
    std::printf("]}\n");
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s input.txt sample_out.bin\n", argv[0]);
        return 2;
    }
    try {
        const Input p = read_input(argv[1]);
        if (p.kind == "batch") return run_batch(p, argv[2]);
        const int ne = (int)p.energies.size();
        std::vector<double> sample;
        std::vector<std::vector<double>> ms;
        const bool atmos = p.kind == "atmos";
        if (!atmos && p.kind != "beam") throw std::runtime_error("kind must be atmos or beam");
        const int nc = atmos ? (int)p.cosines.size() : 1;
        if (atmos) {
            // one propagator per neutrino type, as a caller that keeps both resident would
            AtmosCudaPropagatorSingle nu(0, nc, ne), nubar(0, nc, ne);
            AtmosCudaPropagatorSingle* props[2] = {&nu, &nubar};
            for (int t = 0; t < 2; t++) {
                props[t]->setEnergyList(p.energies);
                props[t]->setCosineList(p.cosines);
                props[t]->setMNSMatrix(p.t12, p.t13, p.t23, p.dcp, t == 0 ? 1 : -1);
                props[t]->setNeutrinoMasses(p.dm12, p.dm23);
                props[t]->setDensity(p.radii, p.rhos, p.yes);
                props[t]->setProductionHeight(p.height);
            }
            for (int w = 0; w < p.warmup; w++)
                for (int t = 0; t < 2; t++) call_ms(*props[t], t == 0 ? Neutrino : Antineutrino);
            for (int s = 0; s < p.steps; s++) {
                std::vector<double> one;
                for (int t = 0; t < 2; t++) one.push_back(call_ms(*props[t], t == 0 ? Neutrino : Antineutrino));
                ms.push_back(one);
            }
            for (int t = 0; t < 2; t++)
                for (int ic = 0; ic < nc; ic += p.sample_every)
                    for (int ie = 0; ie < ne; ie++)
                        for (int c = 0; c < 9; c++) sample.push_back(props[t]->getProbability(ic, ie, ProbType(c)));
        } else {
            BeamCudaPropagatorSingle nu(0, ne, 1), nubar(0, ne, 1);
            BeamCudaPropagatorSingle* props[2] = {&nu, &nubar};
            for (int t = 0; t < 2; t++) {
                props[t]->setEnergyList(p.energies);
                props[t]->setMNSMatrix(p.t12, p.t13, p.t23, p.dcp, t == 0 ? 1 : -1);
                props[t]->setNeutrinoMasses(p.dm12, p.dm23);
                props[t]->setDensity(p.rho);
                props[t]->setPathLength(p.length);
            }
            for (int w = 0; w < p.warmup; w++)
                for (int t = 0; t < 2; t++) call_ms(*props[t], t == 0 ? Neutrino : Antineutrino);
            for (int s = 0; s < p.steps; s++) {
                std::vector<double> one;
                for (int t = 0; t < 2; t++) one.push_back(call_ms(*props[t], t == 0 ? Neutrino : Antineutrino));
                ms.push_back(one);
            }
            for (int t = 0; t < 2; t++)
                for (int ie = 0; ie < ne; ie++)
                    for (int c = 0; c < 9; c++) sample.push_back(props[t]->getProbability(ie, ProbType(c)));
        }
        FILE* f = std::fopen(argv[2], "wb");
        if (!f) throw std::runtime_error("cannot write the sample file");
        const size_t wrote = std::fwrite(sample.data(), sizeof(double), sample.size(), f);
        std::fclose(f);
        if (wrote != sample.size()) throw std::runtime_error("short write of the sample file");
        cudaDeviceProp prop;
        cudaGetDeviceProperties(&prop, 0);
        std::printf("{\"kind\": \"%s\", \"device\": \"%s\", \"n_cosines\": %d, \"n_energies\": %d, "
                    "\"sample_every\": %d, \"ms_per_call\": [",
                    p.kind.c_str(), prop.name, nc, ne, atmos ? p.sample_every : 1);
        for (size_t s = 0; s < ms.size(); s++)
            std::printf("%s[%.6f, %.6f]", s ? ", " : "", ms[s][0], ms[s][1]);
        std::printf("]}\n");
        return 0;
    } catch (const std::exception& e) {
        std::printf("{\"error\": \"%s\"}\n", e.what());
        return 3;
    }
}

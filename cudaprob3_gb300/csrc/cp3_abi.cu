// cp3_abi.cu -- the C ABI (include/cudaprob3_gb300.h): handle state, validation, device
// buffers, launches and result access.
//
// State that the reference keeps in process globals and __constant__ symbols
// (physics.hpp:115-125) is per handle here: the oscillation block travels by value as a
// kernel parameter and everything else lives in the handle's own device buffers, so handles
// never interfere.  Uploads happen lazily at compute time and only for what changed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cudaprob3_gb300.h"
#include "cp3_host.hpp"
#include "cp3_kernels.hpp"
#include "cp3_trace.hpp"

using namespace cp3;

namespace {

thread_local std::string g_create_error;

template <class T>
struct DevBuf {
    T* ptr = nullptr;
    size_t count = 0;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    // Grows to at least n elements (contents not kept).
    cudaError_t reserve(size_t n) {
        if (n <= count && ptr) return cudaSuccess;
        release();
        const cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) {
            ptr = nullptr;
            return e;
        }
        count = n;
        return cudaSuccess;
    }
};

}  // namespace

struct cp3_propagator {
    int kind = 0;  // 0 atmospheric, 1 beam
    int device = 0, nc = 0, ne = 0, precision = CP3_FP64;
    cudaStream_t stream = nullptr;
    cudaStream_t last_stream = nullptr;  // stream of the last compute: results are read after it
    std::string err;

    MixingInput mix;
    bool mns_set = false, masses_set = false;
    std::vector<double> cosines;  // the host builds the trajectories from it
    bool energies_set = false, cosines_set = false;
    EarthModel model;
    bool model_set = false;
    double height_cm = 0.0;
    bool height_set = false;
    double beam_rho = 0.0, beam_L = 0.0;
    bool beam_rho_set = false, beam_L_set = false;
    int avg_bins = 0;
    std::vector<double> avg_prob, avg_edges;

    TrajectoryTable traj;
    bool traj_dirty = true;
    int ncls_used = 0;

    DevBuf<double> d_energies;
    DevBuf<float2> d_energies_df, d_cls_rho_df;  // mixed kernels: (hi, lo) pairs split here
    DevBuf<int> d_seg_off;
    DevBuf<double> d_seg_len, d_cls_rho, d_seg_rho;
    DevBuf<double> d_ph_prob, d_ph_shift, d_air_cm;  // production-height averaging (FP64)
    DevBuf<float> d_ph_prob_f, d_ph_hw;              // ... and its float form (mixed)
    DevBuf<float2> d_ph_hm;
    bool avg_dirty = true;
    DevBuf<float2> d_seg_len_df;
    DevBuf<double> d_table64;
    DevBuf<double> d_plane;  // getProbabilityArr: one channel, transposed on the device
    DevBuf<float> d_table32;
    DevBuf<char> d_result;
    size_t result_bytes = 0;

    void* h_result = nullptr;  // pinned, lazily allocated: the device result's layout and type
    bool result_on_host = false;
    bool computed = false;

    bool profiling = false;
    bool timed = false;
    bool timed_table = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    // Energy lists go up asynchronously on `stream` from two pinned staging slots used in
    // turn (ev_stage[i] marks the end of slot i's last upload, so a setter waits only for the
    // upload two calls back, not for the last compute the newest upload is queued behind); a
    // compute on another stream waits for ev_upload.  ev_done marks the end of the last
    // compute (on last_stream): uploads and computes that overwrite what it reads or writes
    // wait for it.
    cudaEvent_t ev_done = nullptr, ev_upload = nullptr;
    bool upload_pending = false;
    void* h_stage = nullptr;  // 2 x ne doubles
    cudaEvent_t ev_stage[2] = {nullptr, nullptr};
    bool stage_busy[2] = {false, false};
    int stage_slot = 0;

    // The downloads of calculate_to_host_async (atmospheric row pieces) run on copy_stream:
    // piece c's copy waits for ev_piece[c] (its rows computed) and records
    // ev_piece_copied[c]; ev_copied marks the end of the last download.  A later compute of
    // the same row pieces waits for each piece's copy only, so it can run while the rest of
    // the download is on the link; any other compute waits for the whole download.
    // copy_rows: the row cuts of the last download (empty: none issued).
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> ev_piece, ev_piece_copied;
    cudaEvent_t ev_copied = nullptr;
    std::vector<int> copy_rows;

    ~cp3_propagator() {
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (cudaEvent_t& e : ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_piece) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_piece_copied) cudaEventDestroy(e);
        if (ev_copied) cudaEventDestroy(ev_copied);
        if (ev_done) cudaEventDestroy(ev_done);
        if (ev_upload) cudaEventDestroy(ev_upload);
        for (cudaEvent_t e : ev_stage)
            if (e) cudaEventDestroy(e);
        if (h_stage) cudaFreeHost(h_stage);
        if (h_result) cudaFreeHost(h_result);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// Pieces of a pipelined compute-and-copy: enough to hide most of the computation behind the
// copy, few enough that each piece's kernel still fills the GPU.  A piece moves at least
// kMinChunkBytes: below that a piece's kernel launch and copy set-up cost more than the
// overlap gains (a 400 x 400 grid, 5.8 MB per type, goes down in one piece).
constexpr int kDefaultCopyChunks = 4;
constexpr size_t kMinChunkBytes = size_t(32) << 20;

// x[i] as float pairs (hi, lo), hi + lo = x[i] to ~48 bits (the device's df_from, done once).
void split_pairs(const double* x, size_t n, float2* out) {
    for (size_t i = 0; i < n; i++) {
        const float h = (float)x[i];
        out[i] = make_float2(h, (float)(x[i] - (double)h));
    }
}
std::vector<float2> split_pairs(const double* x, size_t n) {
    std::vector<float2> out(n);
    split_pairs(x, n, out.data());
    return out;
}

int fail(cp3_propagator* h, int code, const std::string& msg) {
    if (h)
        h->err = msg;
    else
        g_create_error = msg;
    return code;
}

int cuda_fail(cp3_propagator* h, cudaError_t e, const char* where) {
    cudaGetLastError();  // clear a sticky-free error so the handle stays usable
    return fail(h, e == cudaErrorMemoryAllocation ? CP3_ERR_OOM : CP3_ERR_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}

#define CP3_CUDA(h, call, where)                            \
    do {                                                    \
        const cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, where); \
    } while (0)

int check_handle(cp3_propagator* h) {
    if (!h) return fail(nullptr, CP3_ERR_BAD_ARGUMENT, "null propagator handle");
    return CP3_OK;
}

int create(int kind, int device, int nc, int ne, int precision, cp3_propagator** out) {
    if (!out) return fail(nullptr, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (precision != CP3_FP64 && precision != CP3_MIXED)
        return fail(nullptr, CP3_ERR_BAD_ARGUMENT, "unknown precision");
    if (ne <= 0 || (kind == 0 && nc <= 0))
        return fail(nullptr, CP3_ERR_BAD_SIZE, "grid sizes must be positive");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, CP3_ERR_CUDA, "No GPU found");
    }
    if (device < 0 || device >= ndev)
        return fail(nullptr, CP3_ERR_BAD_ARGUMENT,
                    "The requested GPU Id " + std::to_string(device) + " is not available.");
    cp3_propagator* h = new cp3_propagator();
    h->kind = kind;
    h->device = device;
    h->nc = kind == 0 ? nc : 1;
    h->ne = ne;
    h->precision = precision;
    if (kind == 0) h->cosines.assign(nc, 0.0);
    const size_t elems = (size_t)9 * h->nc * ne;
    h->result_bytes = elems * (precision == CP3_FP64 ? sizeof(double) : sizeof(float));
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_upload, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_stage[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_stage[1], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMallocHost(&h->h_stage, 2 * (size_t)ne * sizeof(double))) != cudaSuccess ||
        (e = h->d_energies.reserve(ne)) != cudaSuccess ||
        (precision == CP3_MIXED && (e = h->d_energies_df.reserve(ne)) != cudaSuccess) ||
        (e = h->d_result.reserve(h->result_bytes)) != cudaSuccess) {
        cudaGetLastError();
        const std::string msg = std::string("propagator creation failed: ") + cudaGetErrorString(e);
        delete h;
        return fail(nullptr, e == cudaErrorMemoryAllocation ? CP3_ERR_OOM : CP3_ERR_CUDA, msg);
    }
    *out = h;
    return CP3_OK;
}

// The host-synchronous uploads and reallocations below overwrite what the last compute
// reads: they start once it has ended.
int wait_last_compute(cp3_propagator* h) {
    if (h->last_stream) CP3_CUDA(h, cudaEventSynchronize(h->ev_done), "wait for the last compute");
    if (!h->copy_rows.empty()) CP3_CUDA(h, cudaEventSynchronize(h->ev_copied), "wait for the last download");
    return CP3_OK;
}

// The copy stream and n piece events of calculate_to_host_async, made on first use.
cudaError_t ensure_copy_events(cp3_propagator* h, int n) {
    cudaError_t e = cudaSuccess;
    if (!h->copy_stream) {
        e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_copied, cudaEventDisableTiming);
    }
    while (e == cudaSuccess && (int)h->ev_piece.size() < n) {
        cudaEvent_t a = nullptr, b = nullptr;
        e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
        if (e != cudaSuccess) break;
        e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            break;
        }
        h->ev_piece.push_back(a);
        h->ev_piece_copied.push_back(b);
    }
    return e;
}

// Uploads the trajectory table and density classes if any of their inputs changed.
int prepare_atmos(cp3_propagator* h) {
    if (!h->traj_dirty) return CP3_OK;
    if (int rc = wait_last_compute(h)) return rc;
    std::string msg;
    int rc = build_trajectories(h->model, h->cosines.data(), h->nc, h->height_cm, &h->traj, &msg);
    if (rc) return fail(h, rc, msg);
    const TrajectoryTable& t = h->traj;
    const size_t nseg = t.len_km.size();
    CP3_CUDA(h, h->d_seg_off.reserve(t.offset.size()), "allocate trajectories");
    CP3_CUDA(h, cudaMemcpy(h->d_seg_off.ptr, t.offset.data(), sizeof(int) * t.offset.size(),
                           cudaMemcpyHostToDevice), "upload trajectories");
    if (h->precision == CP3_FP64) {
        CP3_CUDA(h, h->d_seg_len.reserve(nseg), "allocate trajectories");
        CP3_CUDA(h, cudaMemcpy(h->d_seg_len.ptr, t.len_km.data(), sizeof(double) * nseg,
                               cudaMemcpyHostToDevice), "upload trajectories");
    } else {
        const std::vector<float2> df = split_pairs(t.len_km.data(), nseg);
        CP3_CUDA(h, h->d_seg_len_df.reserve(nseg), "allocate trajectories");
        CP3_CUDA(h, cudaMemcpy(h->d_seg_len_df.ptr, df.data(), sizeof(float2) * nseg,
                               cudaMemcpyHostToDevice), "upload trajectories");
    }
    if (h->model.poly) {  // per-segment densities, no classes or eigen table
        CP3_CUDA(h, h->d_seg_rho.reserve(nseg), "allocate trajectories");
        CP3_CUDA(h, cudaMemcpy(h->d_seg_rho.ptr, t.rho_e.data(), sizeof(double) * nseg,
                               cudaMemcpyHostToDevice), "upload trajectories");
        h->traj_dirty = false;
        return CP3_OK;
    }
    // density classes: 0 = air, 1 + i = shell i (getDensityOfLayer: rhos[i] * yps[i])
    h->ncls_used = 1 + *std::max_element(t.maxlayers.begin(), t.maxlayers.end());
    std::vector<double> cls_rho(h->ncls_used, 0.0);
    for (int c = 1; c < h->ncls_used; c++) cls_rho[c] = h->model.rho[c - 1] * h->model.ye[c - 1];
    CP3_CUDA(h, h->d_cls_rho.reserve(cls_rho.size()), "allocate classes");
    CP3_CUDA(h, cudaMemcpy(h->d_cls_rho.ptr, cls_rho.data(), sizeof(double) * cls_rho.size(),
                           cudaMemcpyHostToDevice), "upload classes");
    if (h->precision == CP3_MIXED) {
        const std::vector<float2> pairs = split_pairs(cls_rho.data(), cls_rho.size());
        CP3_CUDA(h, h->d_cls_rho_df.reserve(pairs.size()), "allocate classes");
        CP3_CUDA(h, cudaMemcpy(h->d_cls_rho_df.ptr, pairs.data(), sizeof(float2) * pairs.size(),
                               cudaMemcpyHostToDevice), "upload classes");
    }
    const size_t cells = (size_t)h->ncls_used * pad_energies(h->ne);
    if (h->precision == CP3_FP64)
        CP3_CUDA(h, h->d_table64.reserve(cells * kF64Fields), "allocate eigen table");
    else
        CP3_CUDA(h, h->d_table32.reserve(cells * kMixFields), "allocate eigen table");
    h->traj_dirty = false;
    return CP3_OK;
}

// Averaging inputs: the client's probabilities and, per cosine, the path-length shifts at the
// bin edges and the air segment in cm (the reference's `dist` of layer 0).
int prepare_averaging(cp3_propagator* h, AvgArrays* av, AvgMixed* avm) {
    if (h->avg_bins == 0) return CP3_OK;
    if (h->avg_dirty)
        if (int rc = wait_last_compute(h)) return rc;
    if (h->avg_dirty && h->precision == CP3_MIXED) {
        // float probabilities; per (cosine, bin) the mid shift as a float pair and the width,
        // both in km (the phase rates are per km); zero where the air segment is zero, as the
        // reference's d0 = 0 there (physics.hpp:1030-1034)
        std::vector<double> shifts;
        production_height_shifts(h->cosines.data(), h->nc, h->height_cm, h->avg_edges.data(),
                                  h->avg_bins, &shifts);
        const int nb = h->avg_bins;
        std::vector<float> prob(h->avg_prob.begin(), h->avg_prob.end()), hw((size_t)h->nc * nb);
        std::vector<float2> hm((size_t)h->nc * nb);
        for (int ic = 0; ic < h->nc; ic++)
            for (int b = 0; b < nb; b++) {
                const double h0 = shifts[(size_t)ic * (nb + 1) + b], h1 = shifts[(size_t)ic * (nb + 1) + b + 1];
                const bool zero = h->traj.air_cm[ic] == 0.0;
                const double mid_km = zero ? 0.0 : 0.5 * (h1 + h0) / kKm2Cm;
                const float mh = (float)mid_km;
                hm[(size_t)ic * nb + b] = make_float2(mh, (float)(mid_km - (double)mh));
                hw[(size_t)ic * nb + b] = zero ? 0.0f : (float)((h1 - h0) / kKm2Cm);
            }
        CP3_CUDA(h, h->d_ph_prob_f.reserve(prob.size()), "allocate averaging");
        CP3_CUDA(h, h->d_ph_hm.reserve(hm.size()), "allocate averaging");
        CP3_CUDA(h, h->d_ph_hw.reserve(hw.size()), "allocate averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_ph_prob_f.ptr, prob.data(), sizeof(float) * prob.size(),
                               cudaMemcpyHostToDevice), "upload averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_ph_hm.ptr, hm.data(), sizeof(float2) * hm.size(),
                               cudaMemcpyHostToDevice), "upload averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_ph_hw.ptr, hw.data(), sizeof(float) * hw.size(),
                               cudaMemcpyHostToDevice), "upload averaging");
        h->avg_dirty = false;
    }
    if (h->precision == CP3_MIXED) {
        avm->prob = h->d_ph_prob_f.ptr;
        avm->hm = h->d_ph_hm.ptr;
        avm->hw = h->d_ph_hw.ptr;
        avm->nb = h->avg_bins;
        return CP3_OK;
    }
    if (h->avg_dirty) {
        std::vector<double> shifts;
        production_height_shifts(h->cosines.data(), h->nc, h->height_cm, h->avg_edges.data(),
                                 h->avg_bins, &shifts);
        CP3_CUDA(h, h->d_ph_prob.reserve(h->avg_prob.size()), "allocate averaging");
        CP3_CUDA(h, h->d_ph_shift.reserve(shifts.size()), "allocate averaging");
        CP3_CUDA(h, h->d_air_cm.reserve(h->nc), "allocate averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_ph_prob.ptr, h->avg_prob.data(), sizeof(double) * h->avg_prob.size(),
                               cudaMemcpyHostToDevice), "upload averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_ph_shift.ptr, shifts.data(), sizeof(double) * shifts.size(),
                               cudaMemcpyHostToDevice), "upload averaging");
        CP3_CUDA(h, cudaMemcpy(h->d_air_cm.ptr, h->traj.air_cm.data(), sizeof(double) * h->nc,
                               cudaMemcpyHostToDevice), "upload averaging");
        h->avg_dirty = false;
    }
    av->prob = h->d_ph_prob.ptr;
    av->shift = h->d_ph_shift.ptr;
    av->air_cm = h->d_air_cm.ptr;
    av->n_bins = h->avg_bins;
    return CP3_OK;
}

// One computation on stream s.  With host_dst, the result is also copied to host memory:
// atmospheric rows in n_chunks pieces, each piece's copy queued right after its kernel, so
// the copy of one piece overlaps the computation of the next.
int launch(cp3_propagator* h, int type, cudaStream_t s, void* host_dst = nullptr, int n_chunks = 1) {
    TraceRange trace(host_dst ? "calculate_to_host" : "calculate");
    if (type != CP3_NEUTRINO && type != CP3_ANTINEUTRINO)
        return fail(h, CP3_ERR_BAD_ARGUMENT, "neutrino type must be Neutrino or Antineutrino");
    if (!h->energies_set) return fail(h, CP3_ERR_NOT_SET, "energy list was not set");
    if (!h->mns_set) return fail(h, CP3_ERR_NOT_SET, "mixing matrix was not set (setMNSMatrix)");
    if (!h->masses_set)
        return fail(h, CP3_ERR_NOT_SET, "mass differences were not set (setNeutrinoMasses)");
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    OscParams p;
    build_osc_params(h->mix, type == CP3_ANTINEUTRINO, &p);
    cudaError_t e = cudaSuccess;
    // the energies' upload, and the last compute (one result buffer per handle), come first
    if (h->upload_pending && s != h->stream) e = cudaStreamWaitEvent(s, h->ev_upload, 0);
    if (e == cudaSuccess && h->last_stream && h->last_stream != s)
        e = cudaStreamWaitEvent(s, h->ev_done, 0);
    // the rows of the last download: its row pieces wait for their own copies (below), any
    // other compute for all of it
    const bool pieces = host_dst && h->kind == 0;
    if (e == cudaSuccess && !pieces && !h->copy_rows.empty()) e = cudaStreamWaitEvent(s, h->ev_copied, 0);
    if (e != cudaSuccess) return cuda_fail(h, e, "order compute");
    h->timed = false;
    const bool profile = h->profiling && !host_dst;  // kernel times only without copies
    auto mark = [&](int i) {
        if (profile && e == cudaSuccess) e = cudaEventRecord(h->ev[i], s);
    };
    const size_t esz = h->precision == CP3_FP64 ? sizeof(double) : sizeof(float);
    if (h->kind == 0) {
        if (!h->model_set) return fail(h, CP3_ERR_NOT_SET, "density model was not set");
        if (!h->height_set)
            return fail(h, CP3_ERR_NOT_SET,
                        "CudaPropagatorSingle::calculateProbabilities. production height was not set");
        const bool traj_was_dirty = h->traj_dirty;
        int rc = prepare_atmos(h);
        if (rc) return rc;
        if (traj_was_dirty) h->avg_dirty = true;
        AvgArrays av;
        AvgMixed avm;
        rc = prepare_averaging(h, &av, &avm);
        if (rc) return rc;
        mark(0);
        const bool mixed = h->precision == CP3_MIXED;
        if (!h->model.poly) {
            if (mixed)
                e = launch_table_mixed(p, h->d_energies_df.ptr, h->ne, h->d_cls_rho_df.ptr,
                                       h->ncls_used, h->d_table32.ptr, s);
            else
                e = launch_table_f64(p, h->d_energies.ptr, h->ne, h->d_cls_rho.ptr, h->ncls_used,
                                     h->d_table64.ptr, s);
        }
        mark(1);
        auto bins = [&](RowRange rr) {
            if (h->model.poly && mixed && avm.nb > 0)
                return launch_atmos_mixed_inline_avg(p, h->d_energies.ptr, h->ne, h->d_seg_off.ptr,
                                                     h->d_seg_len_df.ptr, h->d_seg_rho.ptr, h->nc,
                                                     avm, (float*)h->d_result.ptr, s, rr);
            if (h->model.poly)
                return launch_atmos_inline(p, mixed, h->d_energies.ptr, h->ne, h->d_seg_off.ptr,
                                           mixed ? (const void*)h->d_seg_len_df.ptr
                                                 : (const void*)h->d_seg_len.ptr,
                                           h->d_seg_rho.ptr, h->nc, av, h->d_result.ptr, s, rr);
            if (mixed && avm.nb > 0)
                return launch_atmos_mixed_avg(p, h->d_table32.ptr, h->ne, h->d_seg_off.ptr,
                                              h->d_seg_len_df.ptr, h->nc, avm,
                                              (float*)h->d_result.ptr, s, rr);
            if (mixed)
                return launch_atmos_mixed(p, h->d_table32.ptr, h->ne, h->d_seg_off.ptr,
                                          h->d_seg_len_df.ptr, h->nc,
                                          (float*)h->d_result.ptr, s, rr);
            return launch_atmos_f64(p, h->d_energies.ptr, h->ne, h->d_table64.ptr,
                                    h->d_seg_off.ptr, h->d_seg_len.ptr, h->nc,
                                    av, (double*)h->d_result.ptr, s, rr);
        };
        if (!host_dst) {
            if (e == cudaSuccess) e = bins(RowRange{});
        } else {
            // each piece: rows [r0, r1) of all 9 channel planes, one 2-D copy on the copy
            // stream once the piece is computed.  The first piece is half the size of the
            // others, so that the link starts sooner (measured 1.5 % off the 59-shell
            // 2000 x 2000 step against equal pieces).
            const int chunks = std::max(1, std::min(n_chunks, h->nc));
            const size_t plane = (size_t)h->nc * h->ne * esz, row = (size_t)h->ne * esz;
            const long long den = 2LL * chunks - 1;
            std::vector<int> cuts{0};
            for (int c = 0; c < chunks; c++) {
                const int r1 = (int)((long long)h->nc * (2 * c + 1) / den);
                if (r1 > cuts.back()) cuts.push_back(r1);
            }
            const int np = (int)cuts.size() - 1;
            if (e == cudaSuccess) e = ensure_copy_events(h, np);
            // the same row pieces as the last download: each waits for its own copy
            const bool same = cuts == h->copy_rows;
            if (e == cudaSuccess && !same && !h->copy_rows.empty())
                e = cudaStreamWaitEvent(s, h->ev_copied, 0);
            for (int c = 0; c < np && e == cudaSuccess; c++) {
                const int r0 = cuts[c], r1 = cuts[c + 1];
                if (same) e = cudaStreamWaitEvent(s, h->ev_piece_copied[c], 0);
                if (e == cudaSuccess) e = bins(RowRange{r0, r1});
                if (e == cudaSuccess) e = cudaEventRecord(h->ev_piece[c], s);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(h->copy_stream, h->ev_piece[c], 0);
                if (e == cudaSuccess)
                    e = cudaMemcpy2DAsync((char*)host_dst + r0 * row, plane,
                                          h->d_result.ptr + r0 * row, plane, (r1 - r0) * row, 9,
                                          cudaMemcpyDeviceToHost, h->copy_stream);
                if (e == cudaSuccess) e = cudaEventRecord(h->ev_piece_copied[c], h->copy_stream);
            }
            if (e == cudaSuccess) e = cudaEventRecord(h->ev_copied, h->copy_stream);
            if (e == cudaSuccess) h->copy_rows = cuts;
        }
        mark(2);
        h->timed_table = true;
    } else {
        if (!h->beam_rho_set) return fail(h, CP3_ERR_NOT_SET, "beam density was not set");
        if (!h->beam_L_set) return fail(h, CP3_ERR_NOT_SET, "beam path length was not set");
        // calculate_beam passes density * density_convert() (physics.hpp:1217-1223)
        const double rho_e = h->beam_rho * kDensityConvert;
        mark(1);
        if (h->precision == CP3_FP64)
            e = launch_beam_f64(p, h->d_energies.ptr, h->ne, rho_e, h->beam_L,
                                (double*)h->d_result.ptr, s);
        else
            e = launch_beam_mixed(p, h->d_energies_df.ptr, h->ne, rho_e, h->beam_L,
                                  (float*)h->d_result.ptr, s);
        mark(2);
        if (host_dst && e == cudaSuccess)
            e = cudaMemcpyAsync(host_dst, h->d_result.ptr, h->result_bytes, cudaMemcpyDeviceToHost, s);
        h->timed_table = false;
    }
    if (e == cudaSuccess) e = cudaEventRecord(h->ev_done, s);
    // the caller's stream then waits for the download: work queued behind it sees the host
    // copy (ev_done, the compute's end, orders later uploads and computes of the handle)
    if (e == cudaSuccess && pieces) e = cudaStreamWaitEvent(s, h->ev_copied, 0);
    if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
    h->result_on_host = false;
    h->computed = true;
    h->last_stream = s;
    h->timed = profile;
    return CP3_OK;
}

// The whole result, downloaded once per computation for the host getters.  The mixed
// kernels' floats stay floats and are widened as they are read: widening all of them up
// front cost more than the download (36e6 values per type on a 2000 x 2000 grid).
int fetch_result(cp3_propagator* h) {
    TraceRange trace("fetch_result");
    if (!h->computed) return fail(h, CP3_ERR_NOT_SET, "no probabilities computed yet");
    if (h->result_on_host) return CP3_OK;
    if (!h->h_result) CP3_CUDA(h, cudaMallocHost(&h->h_result, h->result_bytes), "pinned result");
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    CP3_CUDA(h, cudaStreamSynchronize(h->last_stream ? h->last_stream : h->stream), "synchronize");
    CP3_CUDA(h, cudaMemcpy(h->h_result, h->d_result.ptr, h->result_bytes, cudaMemcpyDeviceToHost),
             "copy result");
    h->result_on_host = true;
    return CP3_OK;
}

// Value i of the downloaded result, as a double.
double host_value(const cp3_propagator* h, size_t i) {
    return h->precision == CP3_FP64 ? static_cast<const double*>(h->h_result)[i]
                                    : (double)static_cast<const float*>(h->h_result)[i];
}

int check_type(cp3_propagator* h, int t) {
    if (t < 0 || t > 8) return fail(h, CP3_ERR_BAD_ARGUMENT, "ProbType must be in 0..8");
    return CP3_OK;
}

}  // namespace

extern "C" {

int cp3_atmos_create(int device, int n_cosines, int n_energies, int precision, cp3_propagator** out) {
    return create(0, device, n_cosines, n_energies, precision, out);
}

int cp3_beam_create(int device, int n_energies, int precision, cp3_propagator** out) {
    return create(1, device, 1, n_energies, precision, out);
}

int cp3_destroy(cp3_propagator* h) {
    if (!h) return CP3_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->last_stream && h->last_stream != h->stream) cudaStreamSynchronize(h->last_stream);
    delete h;
    return CP3_OK;
}

const char* cp3_last_error(const cp3_propagator* h) {
    return h ? h->err.c_str() : g_create_error.c_str();
}

int cp3_get_info(const cp3_propagator* h, int* kind, int* precision, int* n_cosines, int* n_energies) {
    if (!h) return fail(nullptr, CP3_ERR_BAD_ARGUMENT, "null propagator handle");
    if (kind) *kind = h->kind;
    if (precision) *precision = h->precision;
    if (n_cosines) *n_cosines = h->kind == 0 ? h->nc : 0;
    if (n_energies) *n_energies = h->ne;
    return CP3_OK;
}

int cp3_set_energies(cp3_propagator* h, const double* energies, int n) {
    if (int rc = check_handle(h)) return rc;
    if (n != h->ne || !energies)
        return fail(h, CP3_ERR_BAD_SIZE,
                    "Propagator::setEnergyList. Propagator was not created for this number of energy nodes");
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    // This staging slot's last upload (two calls back) must have read it.  (One slot would
    // make every call wait for the previous upload, which is queued behind the last compute.)
    const int slot = h->stage_slot;
    if (h->stage_busy[slot]) CP3_CUDA(h, cudaEventSynchronize(h->ev_stage[slot]), "energy upload");
    double* stage = static_cast<double*>(h->h_stage) + (size_t)slot * h->ne;
    std::memcpy(stage, energies, sizeof(double) * n);
    // The upload overwrites what the last compute reads: it waits for it on the device.
    if (h->last_stream && h->last_stream != h->stream)
        CP3_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_done, 0), "order upload");
    CP3_CUDA(h, cudaMemcpyAsync(h->d_energies.ptr, stage, sizeof(double) * n,
                                cudaMemcpyHostToDevice, h->stream), "upload energies");
    CP3_CUDA(h, cudaEventRecord(h->ev_stage[slot], h->stream), "record upload");
    h->stage_busy[slot] = true;
    h->stage_slot = slot ^ 1;
    // the mixed kernels' float pairs, split on the device from the uploaded doubles (the same
    // roundings as the host split: one list crosses the link once)
    if (h->precision == CP3_MIXED)
        CP3_CUDA(h, launch_split_pairs(h->d_energies.ptr, n, h->d_energies_df.ptr, h->stream),
                 "split energies");
    CP3_CUDA(h, cudaEventRecord(h->ev_upload, h->stream), "record upload");
    h->upload_pending = true;
    h->energies_set = true;
    return CP3_OK;
}

int cp3_set_cosines(cp3_propagator* h, const double* cosines, int n) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 0) return fail(h, CP3_ERR_UNSUPPORTED, "beam propagators have no cosine list");
    if (n != h->nc || !cosines)
        return fail(h, CP3_ERR_BAD_SIZE,
                    "Propagator::setCosineList. Propagator was not created for this number of cosine nodes");
    // An unchanged list keeps the trajectories and its layer check, which passed when it was
    // set (a new model is checked against it in set_model); the reference re-derives both
    // every time, with the same result.
    if (h->cosines_set && std::memcmp(h->cosines.data(), cosines, sizeof(double) * n) == 0)
        return CP3_OK;
    if (h->model_set) {  // setMaxlayers runs on every cosine change (atmoscpupropagator.hpp:378)
        for (int i = 0; i < n; i++)
            if (count_shells(h->model, cosines[i]) > kMaxShells)
                return fail(h, CP3_ERR_LAYER_LIMIT, "setMaxlayers : invalid number of maxLayer");
    }
    h->cosines.assign(cosines, cosines + n);
    h->traj_dirty = true;
    h->cosines_set = true;
    return CP3_OK;
}

int cp3_set_mns(cp3_propagator* h, double t12, double t13, double t23, double dcp, int knutype) {
    if (int rc = check_handle(h)) return rc;
    h->mix.theta12 = t12;
    h->mix.theta13 = t13;
    h->mix.theta23 = t23;
    h->mix.dcp = dcp;
    h->mix.knutype = knutype;
    h->mns_set = true;
    return CP3_OK;
}

int cp3_set_masses(cp3_propagator* h, double dm12sq, double dm23sq) {
    if (int rc = check_handle(h)) return rc;
    h->mix.dm12sq = dm12sq;
    h->mix.dm23sq = dm23sq;
    h->masses_set = true;
    return CP3_OK;
}

static int set_model(cp3_propagator* h, const double* radii, const double* c1, const double* c2,
                     const double* c3, const double* ye, int n, bool poly) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 0)
        return fail(h, CP3_ERR_UNSUPPORTED,
                    "beam propagators take setDensity(rho) and setPathLength(L)");
    EarthModel m;
    std::string msg;
    int rc = make_earth_model(radii, c1, c2, c3, ye, n, poly, &m, &msg);
    if (rc) return fail(h, rc, msg);
    if (h->cosines_set)
        for (double c : h->cosines)
            if (count_shells(m, c) > kMaxShells)
                return fail(h, CP3_ERR_LAYER_LIMIT, "setMaxlayers : invalid number of maxLayer");
    h->model = std::move(m);
    h->model_set = true;
    h->traj_dirty = true;
    return CP3_OK;
}

int cp3_set_layers(cp3_propagator* h, const double* radii, const double* rho, const double* ye, int n) {
    return set_model(h, radii, rho, nullptr, nullptr, ye, n, false);
}

int cp3_set_layers_poly(cp3_propagator* h, const double* radii, const double* a, const double* b,
                        const double* c, const double* ye, int n) {
    return set_model(h, radii, a, b, c, ye, n, true);
}

int cp3_set_density_file(cp3_propagator* h, const char* path, double ye_core, double ye_mantle) {
    if (int rc = check_handle(h)) return rc;
    if (!path) return fail(h, CP3_ERR_BAD_ARGUMENT, "null path");
    int ncols = 0;
    std::vector<std::vector<double>> cols;
    std::string msg;
    int rc = parse_model_file(path, &ncols, &cols, &msg);
    if (rc) return fail(h, rc, msg);
    const int n = (int)cols[0].size();
    if (ncols == 2) {
        std::vector<double> ye(n);
        for (int i = 0; i < n; i++) ye[i] = cols[0][i] <= 3480.0 ? ye_core : ye_mantle;
        return set_model(h, cols[0].data(), cols[1].data(), nullptr, nullptr, ye.data(), n, false);
    }
    if (ncols == 3) return set_model(h, cols[0].data(), cols[1].data(), nullptr, nullptr, cols[2].data(), n, false);
    return set_model(h, cols[0].data(), cols[1].data(), cols[2].data(), cols[3].data(), cols[4].data(), n, true);
}

int cp3_get_n_layer_boundaries(cp3_propagator* h, int* n) {
    if (int rc = check_handle(h)) return rc;
    if (!n) return fail(h, CP3_ERR_BAD_ARGUMENT, "null output");
    if (h->kind != 0) return fail(h, CP3_ERR_UNSUPPORTED, "beam propagators have no layer boundaries");
    if (!h->model_set) return fail(h, CP3_ERR_NOT_SET, "density model was not set");
    *n = (int)h->model.radii.size();
    return CP3_OK;
}

int cp3_set_chemical_composition(cp3_propagator* h, const double* ye, int n) {
    if (int rc = check_handle(h)) return rc;
    if (!h->model_set || !ye || (size_t)n != h->model.ye.size())
        return fail(h, CP3_ERR_BAD_SIZE,
                    "CpuPropagator::setChemicalComposition. Size of input list not equal to expectation.");
    // The reference overwrites yps in its internal (descending) order.
    h->model.ye.assign(ye, ye + n);
    h->traj_dirty = true;
    return CP3_OK;
}

int cp3_set_production_height(cp3_propagator* h, double km) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 0) return fail(h, CP3_ERR_UNSUPPORTED, "beam propagators have no production height");
    if (!h->cosines_set) return fail(h, CP3_ERR_NOT_SET, "must set cosine list before production height");
    h->height_cm = km * 100000.0;
    h->height_set = true;
    h->traj_dirty = true;
    return CP3_OK;
}

int cp3_set_beam_density(cp3_propagator* h, double rho) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 1) {
        // AtmosCpuPropagator::setDensity(rho) is a printing dummy (atmoscpupropagator.hpp:347-358)
        return fail(h, CP3_ERR_UNSUPPORTED,
                    "DUMMY FUNCTION: ATMOS class uses setDensity(radii, rhos, yps) or setDensityFromFile");
    }
    h->beam_rho = rho;
    h->beam_rho_set = true;
    return CP3_OK;
}

int cp3_set_beam_path_length(cp3_propagator* h, double km) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 1)
        return fail(h, CP3_ERR_UNSUPPORTED, "DUMMY FUNCTION - ATMOS class calculates PATH LENGTH");
    h->beam_L = km;
    h->beam_L_set = true;
    return CP3_OK;
}

int cp3_set_production_height_averaging(cp3_propagator* h, int n_bins, const double* prob,
                                        const double* edges_km) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 0) return fail(h, CP3_ERR_UNSUPPORTED, "beam propagators have no production height");
    if (n_bins < 0 || n_bins > kMaxProdHeightBins)
        return fail(h, CP3_ERR_BAD_ARGUMENT,
                    "SetNumberOfProductionHeightBinsForAveraging : invalid number of production height bins");
    if (n_bins == 0) {
        h->avg_bins = 0;
        return CP3_OK;
    }
    h->avg_dirty = true;
    if (!prob || !edges_km) return fail(h, CP3_ERR_BAD_ARGUMENT, "null production-height arrays");
    const size_t np = (size_t)n_bins * 2 * 3 * h->ne * h->nc;
    h->avg_prob.assign(prob, prob + np);
    h->avg_edges.assign(edges_km, edges_km + n_bins + 1);
    h->avg_bins = n_bins;
    return CP3_OK;
}

int cp3_calculate(cp3_propagator* h, int type) {
    if (int rc = check_handle(h)) return rc;
    int rc = launch(h, type, h->stream);
    if (rc) return rc;
    CP3_CUDA(h, cudaStreamSynchronize(h->stream), "waitForCompletion");
    return CP3_OK;
}

int cp3_calculate_async(cp3_propagator* h, int type, void* stream) {
    if (int rc = check_handle(h)) return rc;
    return launch(h, type, stream ? (cudaStream_t)stream : h->stream);
}

int cp3_calculate_to_host_async(cp3_propagator* h, int type, void* dst, int n_chunks, void* stream) {
    if (int rc = check_handle(h)) return rc;
    if (!dst) return fail(h, CP3_ERR_BAD_ARGUMENT, "null destination");
    if (n_chunks <= 0)
        n_chunks = (int)std::max<size_t>(1, std::min<size_t>(kDefaultCopyChunks, h->result_bytes / kMinChunkBytes));
    return launch(h, type, stream ? (cudaStream_t)stream : h->stream, dst, n_chunks);
}

int cp3_synchronize(cp3_propagator* h) {
    if (int rc = check_handle(h)) return rc;
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    CP3_CUDA(h, cudaStreamSynchronize(h->stream), "waitForCompletion");
    if (h->last_stream && h->last_stream != h->stream)
        CP3_CUDA(h, cudaStreamSynchronize(h->last_stream), "waitForCompletion");
    return CP3_OK;
}

int cp3_get_probability(cp3_propagator* h, int ic, int ie, int t, double* out) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 0) return fail(h, CP3_ERR_UNSUPPORTED, "use cp3_get_probability_beam for beam propagators");
    if (int rc = check_type(h, t)) return rc;
    if (ic < 0 || ie < 0 || ic >= h->nc || ie >= h->ne)
        return fail(h, CP3_ERR_INDEX, "CudaPropagatorSingle::getProbability. Invalid indices");
    if (!out) return fail(h, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    if (int rc = fetch_result(h)) return rc;
    *out = host_value(h, ((size_t)t * h->nc + ic) * h->ne + ie);
    return CP3_OK;
}

int cp3_get_probability_beam(cp3_propagator* h, int ie, int t, double* out) {
    if (int rc = check_handle(h)) return rc;
    if (h->kind != 1) return fail(h, CP3_ERR_UNSUPPORTED, "use cp3_get_probability for atmospheric propagators");
    if (int rc = check_type(h, t)) return rc;
    if (ie < 0 || ie >= h->ne)
        return fail(h, CP3_ERR_INDEX, "CudaPropagatorSingle::getProbability. Invalid indices");
    if (!out) return fail(h, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    if (int rc = fetch_result(h)) return rc;
    *out = host_value(h, (size_t)t * h->ne + ie);
    return CP3_OK;
}

int cp3_get_probability_arr(cp3_propagator* h, int t, double* out) {
    TraceRange trace("get_probability_arr");
    if (int rc = check_handle(h)) return rc;
    if (int rc = check_type(h, t)) return rc;
    if (!out) return fail(h, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    if (!h->computed) return fail(h, CP3_ERR_NOT_SET, "no probabilities computed yet");
    const size_t cells = (size_t)h->nc * h->ne;
    if (!h->result_on_host) {
        // the reference downloads all nine channels and reorders on the host
        // (atmoscudapropagator.cu:222-257); here the one channel asked for is transposed on
        // the device and only it crosses the link
        CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
        CP3_CUDA(h, h->d_plane.reserve(cells), "allocate");
        cudaStream_t s = h->last_stream ? h->last_stream : h->stream;
        const bool is_float = h->precision == CP3_MIXED;
        const char* src = h->d_result.ptr + (size_t)t * cells * (is_float ? sizeof(float) : sizeof(double));
        const cudaError_t e = launch_plane_transpose(src, is_float, h->nc, h->ne, h->d_plane.ptr, s);
        if (e == cudaSuccess) {
            CP3_CUDA(h, cudaMemcpyAsync(out, h->d_plane.ptr, cells * sizeof(double),
                                        cudaMemcpyDeviceToHost, s), "copy channel");
            CP3_CUDA(h, cudaStreamSynchronize(s), "synchronize");
            return CP3_OK;
        }
        cudaGetLastError();  // a grid beyond the launch limits: reorder on the host instead
    }
    if (int rc = fetch_result(h)) return rc;
    const size_t base = (size_t)t * cells;
    size_t it = 0;
    for (int ie = 0; ie < h->ne; ie++)
        for (int ic = 0; ic < h->nc; ic++) out[it++] = host_value(h, base + (size_t)ic * h->ne + ie);
    return CP3_OK;
}

int cp3_device_result(cp3_propagator* h, const void** ptr, int* is_float, size_t* bytes) {
    if (int rc = check_handle(h)) return rc;
    if (ptr) *ptr = h->d_result.ptr;
    if (is_float) *is_float = h->precision == CP3_MIXED;
    if (bytes) *bytes = h->result_bytes;
    return CP3_OK;
}

int cp3_copy_result_async(cp3_propagator* h, void* dst, void* stream) {
    if (int rc = check_handle(h)) return rc;
    if (!dst) return fail(h, CP3_ERR_BAD_ARGUMENT, "null destination");
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    cudaStream_t s = stream ? (cudaStream_t)stream : (h->last_stream ? h->last_stream : h->stream);
    // on another stream than the last compute's, the copy waits for it on the device
    if (h->last_stream && s != h->last_stream)
        CP3_CUDA(h, cudaStreamWaitEvent(s, h->ev_done, 0), "order copy");
    CP3_CUDA(h, cudaMemcpyAsync(dst, h->d_result.ptr, h->result_bytes, cudaMemcpyDeviceToHost, s),
             "copy result");
    return CP3_OK;
}

int cp3_trajectory_table(const double* radii, const double* c1, const double* c2,
                         const double* c3, const double* ye, int n_radii, int poly,
                         const double* cosines, int n_cosines, double height_km,
                         int* n_segments, int* n_classes, int* seg_offset, double* seg_len_km,
                         double* seg_rho_e, int* seg_class, double* class_rho_e) {
    if (!n_segments || !n_classes || (n_cosines > 0 && !cosines) || n_cosines < 0)
        return fail(nullptr, CP3_ERR_BAD_ARGUMENT, "null size outputs or cosines");
    EarthModel m;
    std::string msg;
    int rc = make_earth_model(radii, c1, c2, c3, ye, n_radii, poly != 0, &m, &msg);
    if (rc) return fail(nullptr, rc, msg);
    TrajectoryTable t;
    rc = build_trajectories(m, cosines, n_cosines, height_km * 100000.0, &t, &msg);
    if (rc) return fail(nullptr, rc, msg);
    const int maxm = n_cosines > 0 ? *std::max_element(t.maxlayers.begin(), t.maxlayers.end()) : 0;
    *n_segments = (int)t.len_km.size();
    *n_classes = poly ? 0 : 1 + maxm;
    if (seg_offset) std::copy(t.offset.begin(), t.offset.end(), seg_offset);
    if (seg_len_km) std::copy(t.len_km.begin(), t.len_km.end(), seg_len_km);
    if (seg_rho_e) std::copy(t.rho_e.begin(), t.rho_e.end(), seg_rho_e);
    if (seg_class) std::copy(t.cls.begin(), t.cls.end(), seg_class);
    if (class_rho_e && !poly) {
        class_rho_e[0] = 0.0;
        for (int c = 1; c <= maxm; c++) class_rho_e[c] = m.rho[c - 1] * m.ye[c - 1];
    }
    return CP3_OK;
}

int cp3_set_profiling(cp3_propagator* h, int enable) {
    if (int rc = check_handle(h)) return rc;
    CP3_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    if (enable)
        for (cudaEvent_t& e : h->ev)
            if (!e) CP3_CUDA(h, cudaEventCreate(&e), "cudaEventCreate");
    h->profiling = enable != 0;
    h->timed = false;
    return CP3_OK;
}

int cp3_kernel_times(cp3_propagator* h, double* eigen_ms, double* bins_ms) {
    if (int rc = check_handle(h)) return rc;
    if (!h->timed) return fail(h, CP3_ERR_NOT_SET, "no profiled compute (cp3_set_profiling first)");
    CP3_CUDA(h, cudaEventSynchronize(h->ev[2]), "cudaEventSynchronize");
    float a = 0.f, b = 0.f;
    if (h->timed_table) CP3_CUDA(h, cudaEventElapsedTime(&a, h->ev[0], h->ev[1]), "elapsed");
    CP3_CUDA(h, cudaEventElapsedTime(&b, h->ev[1], h->ev[2]), "elapsed");
    if (eigen_ms) *eigen_ms = a;
    if (bins_ms) *bins_ms = b;
    return CP3_OK;
}

}  // extern "C"

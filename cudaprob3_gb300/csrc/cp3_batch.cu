// cp3_batch.cu -- many independent propagation problems in one persistent launch.
//
// A batch holds atmospheric problems (one Earth model and production height for the batch,
// each problem with its own cosine and energy grid) and beam problems (own energies, density
// and one or more baselines), each with its own oscillation parameters and neutrino type.
// One run is one or two launches of a persistent kernel, captured once in a CUDA graph:
//
//   * the grid is (SMs x resident blocks); every warp pulls tiles from an atomic counter;
//   * tiles [0, A) build the per-(class, energy) eigen tables of the atmospheric problems,
//     tiles [A, A+B) compute bins: atmospheric tiles are rows_per_tile cosine rows x 32
//     energies, beam tiles are 32 x beam_chunk energies with every baseline of the problem;
//   * split (the default where there are tables): a launch of the table tiles, then a
//     launch of the bin tiles, which reads the finished tables through the read-only path;
//   * single launch: an atmospheric bin tile first waits until its own problem's table
//     tiles are done.  Those tiles were handed out before it by the same counter, so the
//     warps holding them are running and the wait ends; it is bounded all the same (status
//     flag on time-out).  The serving loop uses this form;
//   * everything a run needs -- descriptors, tile prefix sums, parameters -- is in device
//     memory, so the captured graph replays unchanged while parameters change between runs.
//
// The tile shape (rows_per_tile, blocks per SM, beam_chunk) and the split do not change any
// bin's arithmetic: results are bit-identical across them, which lets an autotuner pick by
// timing alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cudaprob3_gb300.h"
#include "cp3_host.hpp"
#include "cp3_kernels.hpp"
#include "cp3_batch_kernel.cuh"
#include "cp3_trace.hpp"

namespace cp3 {
namespace {

using namespace batchk;

template <class T>
struct Buf {
    T* ptr = nullptr;
    size_t n = 0;
    ~Buf() {
        if (ptr) cudaFree(ptr);
    }
    cudaError_t alloc(size_t count) {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
        const cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
        if (v.empty()) return cudaSuccess;
        return cudaMemcpyAsync(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    }
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace
}  // namespace cp3

using namespace cp3;

struct cp3_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int sms = 0;

    EarthModel model;
    bool model_set = false;
    double height_cm = 0.0;

    struct HostProblem {
        int kind = 0;
        std::vector<double> cz, en, L;
        double rho = 0.0;
        MixingInput mix;
        int type = 0;
        bool params_set = false;
    };
    std::vector<HostProblem> hp;
    bool committed = false;

    std::vector<Problem> probs;
    std::vector<long long> out_off;
    size_t out_floats = 0;
    long long total_bins = 0;

    Buf<Problem> d_probs;
    Buf<int> d_astart, d_bstart;
    Buf<Header> d_hdr;
    Buf<OscParams> d_params;
    Buf<int> d_row_off, d_done, d_status;
    Buf<float2> d_energies, d_cls_rho, d_seg_len, d_baselines;
    Buf<float> d_tables, d_out;
    Buf<unsigned int> d_counter;
    OscParams* h_params = nullptr;  // pinned staging
    bool params_dirty = true;

    int rows_per_tile = 2, blocks_per_sm = 0, beam_chunk = 4;
    bool split_tables = true;      // tables and bins as two launches (cp3_batch_set_split_tables)
    bool withhold_tables = false;  // testing aid: cp3_batch_debug_withhold_tables
    long long total_a = 0, total_b = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev_params = nullptr, ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    bool ran = false;  // ev1 marks the end of a run

    // What a run in pieces (cp3_batch_run_to_host) launches directly: the kernel arguments,
    // the problem mix, the grids of the table and bin instances, the bin-tile prefix sums;
    // set by every configure.
    Args args{};
    int kinds = 0, grid_tab = 1, grid_bins = 1;
    std::vector<int> bstart;
    // The copy stream of a run in pieces, an event per piece, and the end of its copies.
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> ev_piece;
    cudaEvent_t ev_copied = nullptr;
    bool downloads = false;  // ev_copied has been recorded

    ~cp3_batch() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        if (graph) cudaGraphExecDestroy(graph);
        for (cudaEvent_t e : {ev_params, ev0, ev1, ev_copied})
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_piece) cudaEventDestroy(e);
        if (h_params) cudaFreeHost(h_params);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

thread_local std::string g_batch_create_error;

int bfail(cp3_batch* b, int code, const std::string& msg) {
    if (b)
        b->err = msg;
    else
        g_batch_create_error = msg;
    return code;
}

int bcuda(cp3_batch* b, cudaError_t e, const char* where) {
    cudaGetLastError();
    return bfail(b, e == cudaErrorMemoryAllocation ? CP3_ERR_OOM : CP3_ERR_CUDA,
                 std::string(where) + ": " + cudaGetErrorString(e));
}

#define B_CUDA(b, call, where)                                  \
    do {                                                        \
        const cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return bcuda(b, e_, where);      \
    } while (0)

using KernelFn = void (*)(Args);

template <int kPhases>
KernelFn kernel_for_phases(int kinds) {
    return kinds == kAtmos  ? batch_kernel<kAtmos, kPhases>
           : kinds == kBeam ? batch_kernel<kBeam, kPhases>
                            : batch_kernel<kBoth, kPhases>;
}

KernelFn kernel_for(int kinds, int phases = kPhaseAll) {
    return phases == kPhaseTables ? kernel_for_phases<kPhaseTables>(kinds)
           : phases == kPhaseBins ? kernel_for_phases<kPhaseBins>(kinds)
                                  : kernel_for_phases<kPhaseAll>(kinds);
}

int occupancy(int kinds, int* blocks, int phases = kPhaseAll) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kernel_for(kinds, phases), kBlock, 0) ==
                   cudaSuccess
               ? 0
               : 1;
}

int batch_kinds(const std::vector<Problem>& probs) {
    bool a = false, b = false;
    for (const Problem& P : probs) (P.kind == 0 ? a : b) = true;
    return launch_kinds(a, b);
}

// Tile counts for the current shape, the device header and the graph.
int configure(cp3_batch* b) {
    const int n = (int)b->probs.size();
    std::vector<long long> a(n + 1, 0), bb(n + 1, 0);
    for (int p = 0; p < n; p++) {
        long long na = 0, nb = 0;
        problem_tiles(b->probs[p], b->rows_per_tile, b->beam_chunk, &na, &nb);
        a[p + 1] = a[p] + na;
        bb[p + 1] = bb[p] + nb;
    }
    if (a[n] + bb[n] > kMaxTiles)
        return bfail(b, CP3_ERR_BAD_SIZE, "batch too large for one launch: split it or use larger tiles");
    b->total_a = a[n];
    b->total_b = bb[n];
    const std::vector<int> ai(a.begin(), a.end()), bi(bb.begin(), bb.end());
    // Withheld tables (a testing aid): no table tile is handed out, so every atmospheric bin
    // tile's bounded wait runs out and the run reports it.
    Header h{n, b->rows_per_tile, b->beam_chunk, b->withhold_tables ? 0 : (int)a[n], (int)bb[n]};
    B_CUDA(b, cudaMemcpyAsync(b->d_astart.ptr, ai.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream), "upload tiles");
    B_CUDA(b, cudaMemcpyAsync(b->d_bstart.ptr, bi.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream), "upload tiles");
    B_CUDA(b, cudaMemcpyAsync(b->d_hdr.ptr, &h, sizeof(Header), cudaMemcpyHostToDevice, b->stream), "upload header");
    B_CUDA(b, cudaStreamSynchronize(b->stream), "configure");

    // Split launches only where there are tables to build; the withheld-tables testing aid
    // exercises the single launch's bounded wait, so it keeps the single launch.
    const bool split = b->split_tables && a[n] > 0 && !b->withhold_tables;
    const int kinds = batch_kinds(b->probs);
    // (a run in pieces launches the table and bin instances separately, split or not)
    int occ = 0, occ_tab = 0, occ_bins = 0;
    if (occupancy(kinds, &occ, split ? kPhaseBins : kPhaseAll) || occ < 1 ||
        occupancy(kinds, &occ_bins, kPhaseBins) || occ_bins < 1 ||
        (a[n] > 0 && (occupancy(kinds, &occ_tab, kPhaseTables) || occ_tab < 1)))
        return bfail(b, CP3_ERR_CUDA, "occupancy query failed");
    const int bps = b->blocks_per_sm > 0 ? std::min(b->blocks_per_sm, occ) : occ;
    const int grid = std::max(1, b->sms * bps);
    // The table launch needs no more warps than it has tiles.
    const long long tab_blocks = (a[n] + kBlock / 32 - 1) / (kBlock / 32);
    const int grid_tab = (int)std::max(1LL, std::min<long long>((long long)b->sms * occ_tab, tab_blocks));
    Args args{b->d_hdr.ptr, b->d_probs.ptr, b->d_astart.ptr, b->d_bstart.ptr, b->d_params.ptr,
              b->d_energies.ptr, b->d_row_off.ptr, b->d_seg_len.ptr,
              b->d_cls_rho.ptr, b->d_baselines.ptr, b->d_tables.ptr, b->d_out.ptr,
              b->d_done.ptr, b->d_counter.ptr, b->d_status.ptr,
              (long long)b->d_tables.n, (long long)b->d_out.n, (long long)b->d_seg_len.n,
              (long long)b->d_energies.n};
    b->args = args;
    b->kinds = kinds;
    b->grid_tab = grid_tab;
    b->grid_bins = std::max(1, b->sms * std::min(bps, occ_bins));
    b->bstart = bi;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaStream_t cs;
    B_CUDA(b, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_counter.ptr, 0, 2 * sizeof(unsigned int), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_done.ptr, 0, sizeof(int) * std::max(n, 1), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_status.ptr, 0, sizeof(int), cs);
    if (e == cudaSuccess && split) {
        kernel_for(kinds, kPhaseTables)<<<grid_tab, kBlock, 0, cs>>>(args);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            kernel_for(kinds, kPhaseBins)<<<grid, kBlock, 0, cs>>>(args);
            e = cudaGetLastError();
        }
    } else if (e == cudaSuccess) {
        kernel_for(kinds)<<<grid, kBlock, 0, cs>>>(args);
        e = cudaGetLastError();
    }
    const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (e2 == cudaSuccess) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return bcuda(b, e, "graph capture");
    return CP3_OK;
}

int commit(cp3_batch* b) {
    const int n = (int)b->hp.size();
    if (n == 0) return bfail(b, CP3_ERR_NOT_SET, "the batch has no problems");
    std::vector<int> row_off;
    std::vector<float2> energies, cls_rho, seg_len, baselines;
    b->probs.assign(n, Problem{});
    b->out_off.assign(n, 0);
    size_t tab = 0, out = 0;
    b->total_bins = 0;
    auto split = [](double x) {
        const float h = (float)x;
        return make_float2(h, (float)(x - (double)h));
    };
    for (int p = 0; p < n; p++) {
        const cp3_batch::HostProblem& H = b->hp[p];
        if (!H.params_set) return bfail(b, CP3_ERR_NOT_SET, "problem " + std::to_string(p) + " has no parameters");
        Problem& P = b->probs[p];
        P.kind = H.kind;
        P.ne = (int)H.en.size();
        P.ne_pad = pad_energies(P.ne);
        P.param = p;
        P.e_off = (long long)energies.size();
        for (double x : H.en) energies.push_back(split(x));
        if (H.kind == 0) {
            if (!b->model_set) return bfail(b, CP3_ERR_NOT_SET, "atmospheric problems need cp3_batch_set_earth first");
            TrajectoryTable t;
            std::string msg;
            int rc = build_trajectories(b->model, H.cz.data(), (int)H.cz.size(), b->height_cm, &t, &msg);
            if (rc) return bfail(b, rc, msg);
            P.nrows = (int)H.cz.size();
            P.ncls = 1 + *std::max_element(t.maxlayers.begin(), t.maxlayers.end());
            P.row_off = (long long)row_off.size();
            const int base = (int)seg_len.size();
            for (int v : t.offset) row_off.push_back(base + v);
            // (segment l of a row is density class l: build_trajectories numbers them so)
            for (size_t i = 0; i < t.len_km.size(); i++) seg_len.push_back(split(t.len_km[i]));
            P.cls_off = (long long)cls_rho.size();
            cls_rho.push_back(split(0.0));
            for (int c = 1; c < P.ncls; c++) cls_rho.push_back(split(b->model.rho[c - 1] * b->model.ye[c - 1]));
            P.tab_off = (long long)tab;
            tab += align_up((size_t)P.ncls * P.ne_pad * kMixFields, 64);
            P.out_off = (long long)out;
            out += align_up((size_t)9 * P.nrows * P.ne, 32);
            b->total_bins += (long long)P.nrows * P.ne;
        } else {
            P.nrows = (int)H.L.size();
            P.row_off = (long long)baselines.size();
            for (double L : H.L) baselines.push_back(split(L));
            const float2 r = split(H.rho * kDensityConvert);
            P.rho_e[0] = r.x;
            P.rho_e[1] = r.y;
            P.out_off = (long long)out;
            out += align_up((size_t)9 * P.nrows * P.ne, 32);
            b->total_bins += (long long)P.nrows * P.ne;
        }
        b->out_off[p] = P.out_off;
    }
    b->out_floats = out;
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    B_CUDA(b, b->d_probs.alloc(n), "allocate");
    B_CUDA(b, b->d_astart.alloc(n + 1), "allocate");
    B_CUDA(b, b->d_bstart.alloc(n + 1), "allocate");
    B_CUDA(b, b->d_hdr.alloc(1), "allocate");
    B_CUDA(b, b->d_params.alloc(n), "allocate");
    B_CUDA(b, b->d_energies.alloc(energies.size()), "allocate");
    B_CUDA(b, b->d_cls_rho.alloc(cls_rho.size()), "allocate");
    B_CUDA(b, b->d_row_off.alloc(row_off.size()), "allocate");
    B_CUDA(b, b->d_seg_len.alloc(seg_len.size()), "allocate");
    B_CUDA(b, b->d_baselines.alloc(baselines.size()), "allocate");
    B_CUDA(b, b->d_tables.alloc(tab), "allocate eigen tables");
    B_CUDA(b, b->d_out.alloc(out), "allocate results");
    B_CUDA(b, b->d_done.alloc(n), "allocate");
    B_CUDA(b, b->d_status.alloc(1), "allocate");
    B_CUDA(b, b->d_counter.alloc(2), "allocate");
    B_CUDA(b, b->d_probs.upload(b->probs, b->stream), "upload");
    B_CUDA(b, b->d_energies.upload(energies, b->stream), "upload");
    B_CUDA(b, b->d_cls_rho.upload(cls_rho, b->stream), "upload");
    B_CUDA(b, b->d_row_off.upload(row_off, b->stream), "upload");
    B_CUDA(b, b->d_seg_len.upload(seg_len, b->stream), "upload");
    B_CUDA(b, b->d_baselines.upload(baselines, b->stream), "upload");
    if (b->h_params) cudaFreeHost(b->h_params);
    b->h_params = nullptr;
    B_CUDA(b, cudaMallocHost(&b->h_params, sizeof(OscParams) * n), "pinned parameters");
    for (int p = 0; p < n; p++) build_osc_params(b->hp[p].mix, b->hp[p].type, b->h_params + p);
    b->params_dirty = true;
    B_CUDA(b, cudaStreamSynchronize(b->stream), "commit");
    b->committed = true;
    return configure(b);
}

int upload_params(cp3_batch* b, cudaStream_t s) {
    if (b->params_dirty) {
        B_CUDA(b, cudaMemcpyAsync(b->d_params.ptr, b->h_params, sizeof(OscParams) * b->probs.size(),
                                  cudaMemcpyHostToDevice, s), "upload parameters");
        B_CUDA(b, cudaEventRecord(b->ev_params, s), "event");
        b->params_dirty = false;
    }
    return CP3_OK;
}

// A run rewrites the parameters and the result arena: on a stream other than the last
// run's, it waits for that run to end and for the last run_to_host's copies, which may still
// be reading them.
int order_after_last_run(cp3_batch* b, cudaStream_t s) {
    if (b->ran) B_CUDA(b, cudaStreamWaitEvent(s, b->ev1, 0), "order run after the last run");
    if (b->downloads) B_CUDA(b, cudaStreamWaitEvent(s, b->ev_copied, 0), "order run after download");
    return CP3_OK;
}

int launch(cp3_batch* b, cudaStream_t s) {
    if (!b->committed) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_commit first");
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    if (int rc = order_after_last_run(b, s)) return rc;
    if (int rc = upload_params(b, s)) return rc;
    B_CUDA(b, cudaEventRecord(b->ev0, s), "event");
    B_CUDA(b, cudaGraphLaunch(b->graph, s), "graph launch");
    B_CUDA(b, cudaEventRecord(b->ev1, s), "event");
    b->timed = b->ran = true;
    return CP3_OK;
}

// Default pieces of a run to host memory: at least 256 MB each, at most kMaxPieces.
constexpr size_t kMinPieceBytes = size_t(256) << 20;
constexpr int kMaxPieces = 8;

// One run with its results copied to host memory: the table tiles, then the bin tiles in
// n_pieces windows of whole problems of about equal result size.  Each window's range of
// the result arena goes to dst on the batch's copy stream as soon as its launch ends, while
// the next window computes; the caller's stream then waits for the last copy.
int run_to_host(cp3_batch* b, float* dst, int n_pieces, cudaStream_t s) {
    if (!b->committed) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_commit first");
    if (!dst) return bfail(b, CP3_ERR_BAD_ARGUMENT, "cp3_batch_run_to_host: null destination");
    if (b->withhold_tables)
        return bfail(b, CP3_ERR_UNSUPPORTED,
                     "cp3_batch_run_to_host: the withheld-tables testing aid runs through cp3_batch_run only");
    if (n_pieces > kMaxPieces)
        return bfail(b, CP3_ERR_BAD_ARGUMENT, "cp3_batch_run_to_host: at most 8 pieces");
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    const int n = (int)b->probs.size();
    if (n_pieces <= 0)
        n_pieces = (int)std::max<size_t>(1, std::min<size_t>(kMaxPieces, b->out_floats * sizeof(float) / kMinPieceBytes));
    n_pieces = std::min(n_pieces, n);
    if (!b->copy_stream)
        B_CUDA(b, cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking), "copy stream");
    if (!b->ev_copied) B_CUDA(b, cudaEventCreateWithFlags(&b->ev_copied, cudaEventDisableTiming), "event");
    while ((int)b->ev_piece.size() < kMaxPieces) {
        cudaEvent_t e = nullptr;
        B_CUDA(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        b->ev_piece.push_back(e);
    }
    // piece boundaries: the first problem whose results start at or past k/n of the arena
    std::vector<int> cut{0};
    for (int k = 1; k < n_pieces; k++) {
        const long long target = (long long)(b->out_floats * (size_t)k / (size_t)n_pieces);
        int p = cut.back() + 1;
        while (p < n && b->out_off[p] < target) p++;
        if (p < n) cut.push_back(p);
    }
    cut.push_back(n);
    if (int rc = order_after_last_run(b, s)) return rc;
    if (int rc = upload_params(b, s)) return rc;
    B_CUDA(b, cudaEventRecord(b->ev0, s), "event");
    // the resets the captured run does, then the launches of its split form
    B_CUDA(b, cudaMemsetAsync(b->d_counter.ptr, 0, 2 * sizeof(unsigned int), s), "reset");
    B_CUDA(b, cudaMemsetAsync(b->d_done.ptr, 0, sizeof(int) * std::max(n, 1), s), "reset");
    B_CUDA(b, cudaMemsetAsync(b->d_status.ptr, 0, sizeof(int), s), "reset");
    if (b->total_a > 0) {
        kernel_for(b->kinds, kPhaseTables)<<<b->grid_tab, kBlock, 0, s>>>(b->args);
        B_CUDA(b, cudaGetLastError(), "table launch");
    }
    for (size_t i = 0; i + 1 < cut.size(); i++) {
        const int p0 = cut[i], p1 = cut[i + 1];
        Args a = b->args;
        a.bin_lo = b->bstart[p0];
        a.bin_hi = b->bstart[p1];
        B_CUDA(b, cudaMemsetAsync(b->d_counter.ptr + 1, 0, sizeof(unsigned int), s), "reset");
        kernel_for(b->kinds, kPhaseBins)<<<b->grid_bins, kBlock, 0, s>>>(a);
        B_CUDA(b, cudaGetLastError(), "bin launch");
        B_CUDA(b, cudaEventRecord(b->ev_piece[i], s), "event");
        const size_t lo = (size_t)b->out_off[p0], hi = p1 < n ? (size_t)b->out_off[p1] : b->out_floats;
        B_CUDA(b, cudaStreamWaitEvent(b->copy_stream, b->ev_piece[i], 0), "order copy");
        B_CUDA(b, cudaMemcpyAsync(dst + lo, b->d_out.ptr + lo, (hi - lo) * sizeof(float), cudaMemcpyDefault,
                                  b->copy_stream), "copy results");
    }
    B_CUDA(b, cudaEventRecord(b->ev1, s), "event");
    B_CUDA(b, cudaEventRecord(b->ev_copied, b->copy_stream), "event");
    b->downloads = true;
    B_CUDA(b, cudaStreamWaitEvent(s, b->ev_copied, 0), "order copies");
    b->timed = b->ran = true;
    return CP3_OK;
}

std::string tune_cache_path() {
    if (const char* p = std::getenv("CP3_TUNE_CACHE")) return p;
    const char* home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/cp3gb300_tune.txt";
}

std::string tune_key(cp3_batch* b) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, b->device);
    long long na = 0, nb = 0;
    for (const Problem& P : b->probs) (P.kind == 0 ? na : nb)++;
    // problem mix and size, bucketed by powers of two
    const int lg = (int)std::log2((double)std::max<long long>(1, b->total_bins));
    std::string name(prop.name);
    std::replace(name.begin(), name.end(), ' ', '_');
    // "w32s": shapes of the warp-tiled kernel with the launch split (entries of other kernels
    // are never matched)
    return "w32s:" + name + ":a" + std::to_string(na > 0) + "b" + std::to_string(nb > 0) + ":bins2^" + std::to_string(lg);
}

}  // namespace

extern "C" {

int cp3_batch_create(int device, cp3_batch** out) {
    if (!out) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bfail(nullptr, CP3_ERR_CUDA, "No GPU found");
    }
    if (device < 0 || device >= ndev)
        return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "The requested GPU Id " + std::to_string(device) + " is not available.");
    cp3_batch* b = new cp3_batch();
    b->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    for (cudaEvent_t* ev : {&b->ev_params, &b->ev0, &b->ev1})
        if (e == cudaSuccess) e = cudaEventCreate(ev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        const std::string msg = std::string("batch creation failed: ") + cudaGetErrorString(e);
        delete b;
        return bfail(nullptr, CP3_ERR_CUDA, msg);
    }
    *out = b;
    return CP3_OK;
}

int cp3_batch_destroy(cp3_batch* b) {
    delete b;
    return CP3_OK;
}

const char* cp3_batch_last_error(const cp3_batch* b) {
    return b ? b->err.c_str() : g_batch_create_error.c_str();
}

int cp3_batch_set_earth(cp3_batch* b, const double* radii, const double* rho, const double* ye,
                        int n, double production_height_km) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (b->committed) return bfail(b, CP3_ERR_UNSUPPORTED, "the batch is committed");
    std::string msg;
    int rc = make_earth_model(radii, rho, nullptr, nullptr, ye, n, false, &b->model, &msg);
    if (rc) return bfail(b, rc, msg);
    b->height_cm = production_height_km * 100000.0;
    b->model_set = true;
    return CP3_OK;
}

int cp3_batch_add_atmos(cp3_batch* b, const double* cosines, int nc, const double* energies,
                        int ne, int* id) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (b->committed) return bfail(b, CP3_ERR_UNSUPPORTED, "the batch is committed");
    if (nc < 1 || ne < 1 || !cosines || !energies) return bfail(b, CP3_ERR_BAD_SIZE, "empty grid");
    if (!b->model_set) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_set_earth before atmospheric problems");
    for (int i = 0; i < nc; i++)
        if (count_shells(b->model, cosines[i]) > kMaxShells)
            return bfail(b, CP3_ERR_LAYER_LIMIT, "setMaxlayers : invalid number of maxLayer");
    cp3_batch::HostProblem H;
    H.kind = 0;
    H.cz.assign(cosines, cosines + nc);
    H.en.assign(energies, energies + ne);
    b->hp.push_back(std::move(H));
    if (id) *id = (int)b->hp.size() - 1;
    return CP3_OK;
}

int cp3_batch_add_beam(cp3_batch* b, const double* energies, int ne, double rho,
                       const double* path_km, int n_baselines, int* id) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (b->committed) return bfail(b, CP3_ERR_UNSUPPORTED, "the batch is committed");
    if (ne < 1 || !energies || n_baselines < 1 || !path_km) return bfail(b, CP3_ERR_BAD_SIZE, "empty grid");
    cp3_batch::HostProblem H;
    H.kind = 1;
    H.en.assign(energies, energies + ne);
    H.L.assign(path_km, path_km + n_baselines);
    H.rho = rho;
    b->hp.push_back(std::move(H));
    if (id) *id = (int)b->hp.size() - 1;
    return CP3_OK;
}

int cp3_batch_set_params(cp3_batch* b, int id, double t12, double t13, double t23, double dcp,
                         int knutype, double dm12sq, double dm23sq, int neutrino_type) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (id < 0 || id >= (int)b->hp.size()) return bfail(b, CP3_ERR_INDEX, "no such problem");
    if (neutrino_type != CP3_NEUTRINO && neutrino_type != CP3_ANTINEUTRINO)
        return bfail(b, CP3_ERR_BAD_ARGUMENT, "neutrino type must be Neutrino or Antineutrino");
    cp3_batch::HostProblem& H = b->hp[id];
    H.mix.theta12 = t12;
    H.mix.theta13 = t13;
    H.mix.theta23 = t23;
    H.mix.dcp = dcp;
    H.mix.knutype = knutype;
    H.mix.dm12sq = dm12sq;
    H.mix.dm23sq = dm23sq;
    H.type = neutrino_type;
    H.params_set = true;
    if (b->committed) {
        // the previous upload from the staging area must have left before it is rewritten
        B_CUDA(b, cudaEventSynchronize(b->ev_params), "event");
        build_osc_params(H.mix, H.type, b->h_params + id);
        b->params_dirty = true;
    }
    return CP3_OK;
}

int cp3_batch_commit(cp3_batch* b) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (b->committed) return CP3_OK;
    TraceRange trace("batch_commit");
    return commit(b);
}

int cp3_batch_set_shape(cp3_batch* b, int rows_per_tile, int blocks_per_sm, int beam_chunk) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (rows_per_tile < 1 || rows_per_tile > kMaxRowsPerTile || blocks_per_sm < 0 || beam_chunk < 1 ||
        beam_chunk > kMaxBeamChunk)
        return bfail(b, CP3_ERR_BAD_ARGUMENT, "shape: rows_per_tile 1..16, blocks_per_sm >= 0, beam_chunk 1..64");
    b->rows_per_tile = rows_per_tile;
    b->blocks_per_sm = blocks_per_sm;
    b->beam_chunk = beam_chunk;
    if (!b->committed) return CP3_OK;
    B_CUDA(b, cudaStreamSynchronize(b->stream), "synchronize");
    return configure(b);
}

int cp3_batch_set_split_tables(cp3_batch* b, int on) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    b->split_tables = on != 0;
    if (!b->committed) return CP3_OK;
    B_CUDA(b, cudaStreamSynchronize(b->stream), "synchronize");
    return configure(b);
}

int cp3_batch_get_split_tables(const cp3_batch* b, int* on) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (on) *on = b->split_tables ? 1 : 0;
    return CP3_OK;
}

int cp3_batch_debug_withhold_tables(cp3_batch* b, int on) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    b->withhold_tables = on != 0;
    if (!b->committed) return CP3_OK;
    B_CUDA(b, cudaStreamSynchronize(b->stream), "synchronize");
    return configure(b);
}

int cp3_batch_get_shape(const cp3_batch* b, int* rows_per_tile, int* blocks_per_sm, int* beam_chunk) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (rows_per_tile) *rows_per_tile = b->rows_per_tile;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    if (beam_chunk) *beam_chunk = b->beam_chunk;
    return CP3_OK;
}

int cp3_batch_run(cp3_batch* b, void* stream) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    TraceRange trace("batch_run");
    return launch(b, stream ? (cudaStream_t)stream : b->stream);
}

int cp3_batch_run_to_host(cp3_batch* b, void* dst, int n_pieces, void* stream) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    TraceRange trace("batch_run_to_host");
    return run_to_host(b, (float*)dst, n_pieces, stream ? (cudaStream_t)stream : b->stream);
}

int cp3_batch_synchronize(cp3_batch* b, double* ms) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    // everything queued on the batch's own stream, result copies included, and the copies of
    // the last run to host memory
    B_CUDA(b, cudaStreamSynchronize(b->stream), "synchronize");
    if (b->downloads) B_CUDA(b, cudaEventSynchronize(b->ev_copied), "synchronize downloads");
    if (!b->timed) return CP3_OK;
    B_CUDA(b, cudaEventSynchronize(b->ev1), "synchronize");
    if (ms) {
        float f = 0.f;
        B_CUDA(b, cudaEventElapsedTime(&f, b->ev0, b->ev1), "elapsed");
        *ms = f;
    }
    int st = 0;
    B_CUDA(b, cudaMemcpy(&st, b->d_status.ptr, sizeof(int), cudaMemcpyDeviceToHost), "status");
    if (st == kStatusWaitLimit)
        return bfail(b, CP3_ERR_CUDA, "batch kernel: eigen tables did not complete (wait limit)");
    if (st == kStatusBounds)
        return bfail(b, CP3_ERR_CUDA, "batch kernel: a device bounds check failed (CP3_DEVICE_CHECKS build)");
    if (st) return bfail(b, CP3_ERR_CUDA, "batch kernel: a tile of a kind the launch was not built for");
    return CP3_OK;
}

int cp3_batch_tune(cp3_batch* b, int use_cache) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (!b->committed) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_commit first");
    TraceRange trace("batch_tune");
    const std::string key = tune_key(b), path = tune_cache_path();
    if (use_cache) {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line)) {
            std::istringstream in(line);
            std::string k;
            int R, bps, bc, sp;
            if (in >> k >> R >> bps >> bc >> sp && k == key) {
                if (int rc = cp3_batch_set_split_tables(b, sp)) return rc;
                return cp3_batch_set_shape(b, R, bps, bc);
            }
        }
    }
    const int kinds = batch_kinds(b->probs);
    bool has_a = false, has_b = false;
    for (const Problem& P : b->probs) (P.kind == 0 ? has_a : has_b) = true;
    struct Shape {
        int rows, bps, bc, split;
    };
    // Only the dimensions the batch's problem kinds use are swept.
    std::vector<int> rows = has_a ? std::vector<int>{1, 2, 4, 8, 16} : std::vector<int>{2};
    std::vector<int> chunks = has_b ? std::vector<int>{1, 4, 16} : std::vector<int>{4};
    std::vector<int> splits = has_a ? std::vector<int>{0, 1} : std::vector<int>{0};
    std::vector<Shape> cand;
    for (int sp : splits) {
        int occ = 0;
        occupancy(kinds, &occ, sp ? kPhaseBins : kPhaseAll);
        std::vector<int> bps = {0};
        if (occ > 1) bps.push_back(std::max(1, occ / 2));
        for (int r : rows)
            for (int bc : chunks)
                for (int k : bps) cand.push_back({r, k, bc, sp});
    }
    double best = 1e30;
    Shape pick = cand[0];
    for (const Shape& s : cand) {
        int rc = cp3_batch_set_split_tables(b, s.split);
        if (!rc) rc = cp3_batch_set_shape(b, s.rows, s.bps, s.bc);
        if (rc) return rc;
        double total = 0;
        for (int it = 0; it < 4; it++) {
            rc = cp3_batch_run(b, nullptr);
            double ms = 0;
            if (!rc) rc = cp3_batch_synchronize(b, &ms);
            if (rc) return rc;
            if (it > 0) total += ms;
        }
        if (total < best) {
            best = total;
            pick = s;
        }
    }
    int rc = cp3_batch_set_split_tables(b, pick.split);
    if (!rc) rc = cp3_batch_set_shape(b, pick.rows, pick.bps, pick.bc);
    if (rc) return rc;
    if (use_cache) {
        std::ofstream f(path, std::ios::app);
        if (f) f << key << " " << pick.rows << " " << pick.bps << " " << pick.bc << " " << pick.split << "\n";
    }
    return CP3_OK;
}

int cp3_batch_result(cp3_batch* b, int id, const float** ptr, size_t* count) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (!b->committed) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_commit first");
    if (id < 0 || id >= (int)b->probs.size()) return bfail(b, CP3_ERR_INDEX, "no such problem");
    const Problem& P = b->probs[id];
    if (ptr) *ptr = b->d_out.ptr + P.out_off;
    if (count) *count = (size_t)9 * P.nrows * P.ne;
    return CP3_OK;
}

int cp3_batch_copy_result(cp3_batch* b, int id, void* dst, void* stream) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    const float* src = nullptr;
    size_t n = 0;
    if (int rc = cp3_batch_result(b, id, &src, &n)) return rc;
    if (!dst) return bfail(b, CP3_ERR_BAD_ARGUMENT, "null destination");
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (b->ran) B_CUDA(b, cudaStreamWaitEvent(s, b->ev1, 0), "order copy after the last run");
    B_CUDA(b, cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDeviceToHost, s), "copy result");
    return CP3_OK;
}

int cp3_batch_result_offset(const cp3_batch* b, int id, size_t* offset) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (!b->committed) return bfail(const_cast<cp3_batch*>(b), CP3_ERR_NOT_SET, "cp3_batch_commit first");
    if (id < 0 || id >= (int)b->probs.size()) return bfail(const_cast<cp3_batch*>(b), CP3_ERR_INDEX, "no such problem");
    if (offset) *offset = (size_t)b->probs[id].out_off;
    return CP3_OK;
}

int cp3_batch_copy_results(cp3_batch* b, size_t first, size_t count, void* dst, void* stream) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (!b->committed) return bfail(b, CP3_ERR_NOT_SET, "cp3_batch_commit first");
    if (!dst) return bfail(b, CP3_ERR_BAD_ARGUMENT, "null destination");
    if (first > b->out_floats || count > b->out_floats - first)
        return bfail(b, CP3_ERR_INDEX, "range beyond the result arena (" +
                                           std::to_string(b->out_floats) + " floats)");
    if (count == 0) return CP3_OK;
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    // on another stream than the last run's, the copy waits for that run on the device
    if (b->ran) B_CUDA(b, cudaStreamWaitEvent(s, b->ev1, 0), "order copy after the last run");
    B_CUDA(b, cudaMemcpyAsync(dst, b->d_out.ptr + first, count * sizeof(float), cudaMemcpyDefault, s),
           "copy results");
    return CP3_OK;
}

size_t cp3_batch_parameter_bytes(void) { return sizeof(OscParams); }

int cp3_batch_info(const cp3_batch* b, int* n_problems, long long* total_bins, size_t* result_bytes,
                   long long* tiles) {
    if (!b) return bfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null batch");
    if (n_problems) *n_problems = (int)b->hp.size();
    if (total_bins) *total_bins = b->total_bins;
    if (result_bytes) *result_bytes = b->out_floats * sizeof(float);
    if (tiles) *tiles = b->total_a + b->total_b;
    return CP3_OK;
}

}  // extern "C"

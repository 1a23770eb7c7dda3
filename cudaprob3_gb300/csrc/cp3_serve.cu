// cp3_serve.cu -- continuous-batching request loop over the persistent many-problem kernel.
//
// Requests (a registered grid + one parameter set + a neutrino type) are submitted from any
// thread and return at once.  A scheduler thread admits queued requests in arrival order
// whenever device memory and a launch slot are free, packs them into one run of the
// persistent kernel (a table launch and a bin launch where there are atmospheric requests),
// and keeps going: a request that arrives while others run joins the next run, which starts
// on the second slot (stream) while the first is still finishing, so work from consecutive
// runs overlaps on the device.  Grids (trajectory tables, energies,
// class densities) are registered once and stay resident; each request's eigen table and
// result live in a device pool until the client releases the request.  A host callback on the
// stream stamps the completion time and the status of every request of a launch: the
// launch's graph clears the kernel's status word first and copies it into page-locked host
// memory last, so the callback reads it without a CUDA call.  A launch whose CUDA calls fail
// fails its own requests (cp3_server_wait reports the error, cp3_server_result refuses the
// result) and no others.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cudaprob3_gb300.h"
#include "cp3_batch_kernel.cuh"
#include "cp3_host.hpp"
#include "cp3_trace.hpp"

using namespace cp3;
using namespace cp3::batchk;

namespace {

using Clock = std::chrono::steady_clock;
int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now().time_since_epoch()).count();
}

constexpr size_t kUnit = 64;  // pool granularity in floats (256 bytes)
constexpr int kServeRows = 2;       // tile shape of the serving launches: cosine rows per tile
constexpr int kServeBeamChunk = 2;  // and 32-energy groups per beam tile
// Launches with atmospheric requests run as a table launch and a bin launch (see
// capture_slot).
constexpr bool kServeSplitTables = true;

// x as a float pair (hi, lo), hi + lo = x to ~48 bits.
float2 split_pair(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

template <class T>
struct DBuf {
    T* ptr = nullptr;
    size_t n = 0;
    ~DBuf() {
        if (ptr) cudaFree(ptr);
    }
    cudaError_t alloc(size_t count) {
        const cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(count, 1) * sizeof(T));
        n = e == cudaSuccess ? count : 0;
        return e;
    }
};
template <class T>
struct HBuf {  // pinned
    T* ptr = nullptr;
    ~HBuf() {
        if (ptr) cudaFreeHost(ptr);
    }
    cudaError_t alloc(size_t n) { return cudaMallocHost(&ptr, std::max<size_t>(n, 1) * sizeof(T)); }
};

struct Template {
    int kind = 0, ne = 0, ne_pad = 0, nrows = 0, ncls = 0;
    long long e_off = 0, row_off = 0, cls_off = 0;
    float rho_e[2] = {0.f, 0.f};  // beam: rho * 0.5 as a float pair
    size_t tab_floats = 0, out_floats = 0;
    long long bins = 0;
};

// First-fit allocator over one device arena, in kUnit-float units.
class Pool {
    std::map<size_t, size_t> free_;  // offset -> length
public:
    void init(size_t units) {
        free_.clear();
        if (units) free_[0] = units;
    }
    bool alloc(size_t units, size_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < units) continue;
            *off = it->first;
            const size_t rest = it->second - units, o = it->first + units;
            free_.erase(it);
            if (rest) free_[o] = rest;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t units) {
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + units == next->first) {
            units += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += units;
                return;
            }
        }
        free_[off] = units;
    }
};

enum { kQueued = 0, kRunning = 1, kDone = 2 };

// A finished request's status: 0, the persistent kernel's status word (kStatusWaitLimit,
// kStatusKind, kStatusBounds), or kReqLaunchFailed when a CUDA call of its launch failed on the
// host side (the message is in cp3_server::launch_error).
constexpr int kReqLaunchFailed = -1;

struct Request {
    uint64_t id = 0;
    int tmpl = 0;
    OscParams params;
    int64_t t_submit = 0, t_start = 0, t_done = 0;
    size_t pool_off = 0, pool_units = 0;
    std::atomic<int> status{0};  // written before state becomes kDone
    std::atomic<int> state{kQueued};
};

struct Slot {
    struct cp3_server* owner = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};  // by launch kinds (1..3)
    DBuf<Problem> d_probs;
    DBuf<int> d_a, d_b;
    DBuf<Header> d_hdr;
    DBuf<OscParams> d_params;
    DBuf<int> d_done, d_status;
    DBuf<unsigned int> d_counter;
    HBuf<Problem> h_probs;
    HBuf<int> h_a, h_b;
    HBuf<Header> h_hdr;
    HBuf<OscParams> h_params;
    HBuf<int> h_status;  // the launch's status word, copied back by the graph's last node
    std::vector<std::shared_ptr<Request>> reqs;
    bool busy = false;
    std::atomic<int> finished{0};
};

}  // namespace

struct cp3_server {
    int device = 0, sms = 0;
    std::string err;
    std::mutex mu;  // requests map, queues, pool, stats
    std::condition_variable cv;
    EarthModel model;
    bool model_set = false;
    double height_cm = 0.0;
    int max_batch = 256;
    long long max_bins = 8000000;
    int64_t aging_ns = 4000000;  // 4 ms
    size_t pool_bytes = 0;

    // registration (host), then resident device arenas
    std::vector<Template> tmpls;
    std::vector<int> h_row_off;
    std::vector<float2> h_energies, h_cls_rho, h_seg_len, h_baselines;
    DBuf<int> d_row_off;
    DBuf<float2> d_energies, d_cls_rho, d_seg_len, d_baselines;
    DBuf<float> d_pool;
    Pool pool;
    Slot slots[2];

    std::unordered_map<uint64_t, std::shared_ptr<Request>> requests;
    // The queue: one FIFO per registered grid (all its requests have the same size), and the
    // grids in increasing size.  Packing a launch touches only the FIFOs' heads and the
    // requests it admits, however deep the queue.
    std::vector<std::deque<std::shared_ptr<Request>>> queues;
    std::vector<int> by_size;
    long long queued = 0;
    uint64_t next_id = 1;
    std::thread loop;
    std::atomic<bool> stop{false};
    bool started = false;
    std::atomic<long long> launches{0}, completed{0};
    std::string launch_error;      // the last failed launch's CUDA error (under mu)
    int debug_fail_launches = 0;   // testing aid: cp3_server_debug_fail_launches (under mu)

    // completion queue for cp3_server_poll: ids in completion order, recorded once a client
    // has called poll (so a server nobody polls keeps no list)
    std::mutex cq_mu;
    std::condition_variable cq_cv;
    std::deque<uint64_t> completions;
    std::atomic<bool> record_completions{false};

    ~cp3_server();
};

namespace {

thread_local std::string g_server_create_error;

int sfail(cp3_server* s, int code, const std::string& msg) {
    if (s)
        s->err = msg;
    else
        g_server_create_error = msg;
    return code;
}

int scuda(cp3_server* s, cudaError_t e, const char* where) {
    cudaGetLastError();
    return sfail(s, e == cudaErrorMemoryAllocation ? CP3_ERR_OOM : CP3_ERR_CUDA,
                 std::string(where) + ": " + cudaGetErrorString(e));
}

#define S_CUDA(s, call, where)                              \
    do {                                                    \
        const cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return scuda(s, e_, where);  \
    } while (0)

// Marks the requests of a launch done with one status and queues them for cp3_server_poll.
void finish_requests(cp3_server* s, const std::vector<std::shared_ptr<Request>>& reqs, int status) {
    const int64_t t = now_ns();
    for (auto& r : reqs) {
        r->t_done = t;
        r->status.store(status);
        r->state.store(kDone);
    }
    s->completed += (long long)reqs.size();
    if (s->record_completions.load()) {
        {
            std::lock_guard<std::mutex> lk(s->cq_mu);
            for (auto& r : reqs) s->completions.push_back(r->id);
        }
        s->cq_cv.notify_all();
    }
}

// Host callback after a slot's launch: every request of the launch is done, with the status
// word the launch's graph copied into page-locked memory before this callback (stream order).
// It takes no lock of the scheduler's: the scheduler may hold cp3_server::mu while it waits.
void CUDART_CB on_launch_done(void* user) {
    Slot* slot = static_cast<Slot*>(user);
    finish_requests(slot->owner, slot->reqs, *slot->h_status.ptr);
    slot->finished.store(1);
    slot->owner->cv.notify_all();
}

const char* status_text(int st) {
    return st == kStatusBounds      ? "batch kernel: a device bounds check failed (CP3_DEVICE_CHECKS build)"
           : st == kStatusWaitLimit ? "batch kernel reported a wait time-out"
           : st == kStatusKind      ? "batch kernel: a tile of a kind the launch was not built for"
                                    : "the launch of this request failed";
}

// Packs queued requests into one launch on `slot`; caller holds s->mu.  Order: requests
// older than the aging limit first (arrival order), then the rest smallest-first, so small
// requests are not stuck behind large ones and large ones cannot starve.  A request is
// admitted only if its table and result fit in the pool (admission by device memory).
// Requests of one grid have one size, so when a grid's oldest request does not fit (pool or
// the launch's bin cap), none of that grid's does, and the grid is passed over.
void launch_slot(cp3_server* s, Slot& slot) {
    TraceRange trace("serve_launch");
    slot.reqs.clear();
    const int64_t now = now_ns();
    const int ng = (int)s->queues.size();
    std::vector<char> blocked(ng, 0);
    long long bins = 0;
    auto admit = [&](int g) {  // the head of grid g's FIFO, if it fits
        const Template& T = s->tmpls[g];
        if (!slot.reqs.empty() && bins + T.bins > s->max_bins) return false;
        const size_t units = (T.tab_floats + T.out_floats) / kUnit;
        size_t off = 0;
        if (!s->pool.alloc(units, &off)) return false;  // waits for releases
        std::shared_ptr<Request> r = std::move(s->queues[g].front());
        s->queues[g].pop_front();
        s->queued--;
        r->pool_off = off;
        r->pool_units = units;
        bins += T.bins;
        slot.reqs.push_back(std::move(r));
        return true;
    };
    // aged requests, oldest first across the grids' heads
    while ((int)slot.reqs.size() < s->max_batch) {
        int g_old = -1;
        for (int g = 0; g < ng; g++)
            if (!blocked[g] && !s->queues[g].empty() &&
                (g_old < 0 || s->queues[g].front()->t_submit < s->queues[g_old].front()->t_submit))
                g_old = g;
        if (g_old < 0 || now - s->queues[g_old].front()->t_submit <= s->aging_ns) break;
        if (!admit(g_old)) blocked[g_old] = 1;
    }
    // then smallest grids first, each in arrival order
    for (int g : s->by_size)
        while (!blocked[g] && !s->queues[g].empty() && (int)slot.reqs.size() < s->max_batch)
            if (!admit(g)) blocked[g] = 1;
    if (slot.reqs.empty()) return;
    const int n = (int)slot.reqs.size();
    long long a = 0, b = 0;
    slot.h_a.ptr[0] = slot.h_b.ptr[0] = 0;
    const int64_t t0 = now_ns();
    for (int i = 0; i < n; i++) {
        Request& r = *slot.reqs[i];
        const Template& T = s->tmpls[r.tmpl];
        Problem P{};
        P.kind = T.kind;
        P.ne = T.ne;
        P.ne_pad = T.ne_pad;
        P.nrows = T.nrows;
        P.ncls = T.ncls;
        P.param = i;
        P.e_off = T.e_off;
        P.row_off = T.row_off;
        P.cls_off = T.cls_off;
        P.tab_off = (long long)(r.pool_off * kUnit);
        P.out_off = P.tab_off + (long long)T.tab_floats;
        P.rho_e[0] = T.rho_e[0];
        P.rho_e[1] = T.rho_e[1];
        slot.h_probs.ptr[i] = P;
        slot.h_params.ptr[i] = r.params;
        long long na = 0, nb = 0;
        problem_tiles(P, kServeRows, kServeBeamChunk, &na, &nb);
        a += na;
        b += nb;
        slot.h_a.ptr[i + 1] = (int)a;  // < kMaxTiles: a launch holds at most max_bins bins
        slot.h_b.ptr[i + 1] = (int)b;  // besides its first request, and requests fit the pool
        r.t_start = t0;
        r.state.store(kRunning);
    }
    *slot.h_hdr.ptr = Header{n, kServeRows, kServeBeamChunk, (int)a, (int)b};
    cudaStream_t st = slot.stream;
    bool has_atmos = false, has_beam = false;
    for (int i = 0; i < n; i++) (slot.h_probs.ptr[i].kind == 0 ? has_atmos : has_beam) = true;
    slot.finished.store(0);
    s->launches++;
    // Every call is checked.  A launch that fails before its host callback is queued fails
    // its own requests here, after its stream has drained (so no kernel of it can still
    // write into pool memory that a release hands to the next request).
    cudaError_t e = cudaSuccess;
    const char* what = "";
    bool graph_queued = false;
    if (s->debug_fail_launches > 0) {
        s->debug_fail_launches--;
        e = cudaErrorLaunchFailure;
        what = "injected launch failure (cp3_server_debug_fail_launches)";
    }
#define SERVE_STEP(call, name)        \
    if (e == cudaSuccess) {           \
        e = (call);                   \
        if (e != cudaSuccess) what = name; \
    }
    SERVE_STEP(cudaMemcpyAsync(slot.d_probs.ptr, slot.h_probs.ptr, sizeof(Problem) * n, cudaMemcpyHostToDevice, st), "upload problems")
    SERVE_STEP(cudaMemcpyAsync(slot.d_params.ptr, slot.h_params.ptr, sizeof(OscParams) * n, cudaMemcpyHostToDevice, st), "upload parameters")
    SERVE_STEP(cudaMemcpyAsync(slot.d_a.ptr, slot.h_a.ptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st), "upload tile offsets")
    SERVE_STEP(cudaMemcpyAsync(slot.d_b.ptr, slot.h_b.ptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st), "upload tile offsets")
    SERVE_STEP(cudaMemcpyAsync(slot.d_hdr.ptr, slot.h_hdr.ptr, sizeof(Header), cudaMemcpyHostToDevice, st), "upload header")
    SERVE_STEP(cudaGraphLaunch(slot.graph[launch_kinds(has_atmos, has_beam)], st), "graph launch")
    graph_queued = e == cudaSuccess;
    SERVE_STEP(cudaLaunchHostFunc(st, on_launch_done, &slot), "completion callback")
#undef SERVE_STEP
    if (e == cudaSuccess) {
        slot.busy = true;
        return;
    }
    cudaGetLastError();
    if (graph_queued) cudaStreamSynchronize(st);
    s->launch_error = std::string("serve launch: ") + what + ": " + cudaGetErrorString(e);
    finish_requests(s, slot.reqs, kReqLaunchFailed);
    slot.reqs.clear();
    s->cv.notify_all();
}

void scheduler(cp3_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop.load()) {
        for (Slot& sl : s->slots) {
            if (sl.busy && sl.finished.load()) {  // the callback has set every request's status
                sl.busy = false;
                sl.reqs.clear();
            }
        }
        bool launched = false;
        for (Slot& sl : s->slots)
            if (!sl.busy && s->queued > 0) {
                launch_slot(s, sl);
                launched = launched || sl.busy;
            }
        // Nothing launchable (slots busy, queue empty, or the pool full until a release):
        // sleep with the mutex released.  No predicate here -- a predicate that is already true
        // would return without releasing it, and release() needs the mutex to free memory.
        // The completion callback notifies without the mutex, so the wait is short.
        if (!launched) s->cv.wait_for(lk, std::chrono::microseconds(20));
    }
}

int capture_slot(cp3_server* s, Slot& sl) {
    const int cap = s->max_batch;
    S_CUDA(s, cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "stream");
    S_CUDA(s, sl.d_probs.alloc(cap), "allocate");
    S_CUDA(s, sl.d_a.alloc(cap + 1), "allocate");
    S_CUDA(s, sl.d_b.alloc(cap + 1), "allocate");
    S_CUDA(s, sl.d_hdr.alloc(1), "allocate");
    S_CUDA(s, sl.d_params.alloc(cap), "allocate");
    S_CUDA(s, sl.d_done.alloc(cap), "allocate");
    S_CUDA(s, sl.d_status.alloc(1), "allocate");
    S_CUDA(s, sl.d_counter.alloc(2), "allocate");
    S_CUDA(s, sl.h_probs.alloc(cap), "pinned");
    S_CUDA(s, sl.h_a.alloc(cap + 1), "pinned");
    S_CUDA(s, sl.h_b.alloc(cap + 1), "pinned");
    S_CUDA(s, sl.h_hdr.alloc(1), "pinned");
    S_CUDA(s, sl.h_params.alloc(cap), "pinned");
    S_CUDA(s, sl.h_status.alloc(1), "pinned");
    *sl.h_status.ptr = 0;
    Args args{sl.d_hdr.ptr, sl.d_probs.ptr, sl.d_a.ptr, sl.d_b.ptr, sl.d_params.ptr,
              s->d_energies.ptr, s->d_row_off.ptr, s->d_seg_len.ptr,
              s->d_cls_rho.ptr, s->d_baselines.ptr, s->d_pool.ptr, s->d_pool.ptr,
              sl.d_done.ptr, sl.d_counter.ptr, sl.d_status.ptr,
              (long long)s->d_pool.n, (long long)s->d_pool.n, (long long)s->d_seg_len.n,
              (long long)s->d_energies.n};
    // One graph per set of problem kinds; a launch replays the one for the kinds it holds.
    // With atmospheric requests it is a table launch, then a bin launch that reads the
    // finished tables (no wait); a beam-only launch is the single kernel.  The table launch
    // has a full grid: the number of table tiles changes from launch to launch, and warps
    // without a tile return at once.  Each graph clears the status word first and copies it
    // to the slot's page-locked word last, where the completion callback reads it.
    for (int kinds = 1; kinds <= 3; kinds++) {
        using Kern = void (*)(Args);
        const bool split = kServeSplitTables && (kinds & kAtmos);
        const Kern tab = kinds == kAtmos ? batch_kernel<kAtmos, kPhaseTables> : batch_kernel<kBoth, kPhaseTables>;
        const Kern kern = !split ? (kinds == kBeam ? batch_kernel<kBeam> : kinds == kAtmos ? batch_kernel<kAtmos>
                                                                                           : batch_kernel<kBoth>)
                                 : (kinds == kAtmos ? batch_kernel<kAtmos, kPhaseBins> : batch_kernel<kBoth, kPhaseBins>);
        int occ = 0, occ_tab = 0;
        S_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kBlock, 0), "occupancy");
        if (split) S_CUDA(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_tab, tab, kBlock, 0), "occupancy");
        const int grid = std::max(1, s->sms * std::max(occ, 1));
        const int grid_tab = std::max(1, s->sms * std::max(occ_tab, 1));
        cudaStream_t cs;
        S_CUDA(s, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_counter.ptr, 0, 2 * sizeof(unsigned int), cs);
        if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_done.ptr, 0, sizeof(int) * cap, cs);
        if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_status.ptr, 0, sizeof(int), cs);
        if (e == cudaSuccess && split) {
            tab<<<grid_tab, kBlock, 0, cs>>>(args);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            kern<<<grid, kBlock, 0, cs>>>(args);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.h_status.ptr, sl.d_status.ptr, sizeof(int), cudaMemcpyDeviceToHost, cs);
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&sl.graph[kinds], g, 0);
        if (e2 == cudaSuccess) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return scuda(s, e, "graph capture");
    }
    return CP3_OK;
}

template <class T>
cudaError_t upload(DBuf<T>& d, const std::vector<T>& v) {
    cudaError_t e = d.alloc(v.size());
    if (e == cudaSuccess && !v.empty())
        e = cudaMemcpy(d.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
    return e;
}

}  // namespace

cp3_server::~cp3_server() {
    stop.store(true);
    cv.notify_all();
    if (loop.joinable()) loop.join();
    cudaSetDevice(device);
    for (Slot& sl : slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        for (cudaGraphExec_t gx : sl.graph)
            if (gx) cudaGraphExecDestroy(gx);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
}

extern "C" {

int cp3_server_create(int device, size_t pool_bytes, int max_batch, long long max_bins_per_launch,
                      cp3_server** out) {
    if (!out) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (max_batch < 1 || max_batch > 65536 || max_bins_per_launch < 1 || pool_bytes < (1u << 20))
        return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "max_batch 1..65536, max_bins >= 1, pool >= 1 MiB");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return sfail(nullptr, CP3_ERR_CUDA, "No GPU found");
    }
    if (device < 0 || device >= ndev)
        return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "The requested GPU Id " + std::to_string(device) + " is not available.");
    cp3_server* s = new cp3_server();
    s->device = device;
    s->max_batch = max_batch;
    s->max_bins = max_bins_per_launch;
    s->pool_bytes = pool_bytes;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
    for (Slot& sl : s->slots) sl.owner = s;
    *out = s;
    return CP3_OK;
}

int cp3_server_destroy(cp3_server* s) {
    delete s;
    return CP3_OK;
}

const char* cp3_server_last_error(const cp3_server* s) {
    return s ? s->err.c_str() : g_server_create_error.c_str();
}

int cp3_server_set_earth(cp3_server* s, const double* radii, const double* rho, const double* ye,
                         int n, double production_height_km) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (s->started) return sfail(s, CP3_ERR_UNSUPPORTED, "the server is running");
    std::string msg;
    int rc = make_earth_model(radii, rho, nullptr, nullptr, ye, n, false, &s->model, &msg);
    if (rc) return sfail(s, rc, msg);
    s->height_cm = production_height_km * 100000.0;
    s->model_set = true;
    return CP3_OK;
}

int cp3_server_add_atmos_grid(cp3_server* s, const double* cosines, int nc, const double* energies,
                              int ne, int* grid) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (s->started) return sfail(s, CP3_ERR_UNSUPPORTED, "the server is running");
    if (!s->model_set) return sfail(s, CP3_ERR_NOT_SET, "cp3_server_set_earth before atmospheric grids");
    if (nc < 1 || ne < 1 || !cosines || !energies) return sfail(s, CP3_ERR_BAD_SIZE, "empty grid");
    TrajectoryTable t;
    std::string msg;
    int rc = build_trajectories(s->model, cosines, nc, s->height_cm, &t, &msg);
    if (rc) return sfail(s, rc, msg);
    Template T;
    T.kind = 0;
    T.ne = ne;
    T.ne_pad = pad_energies(ne);
    T.nrows = nc;
    T.ncls = 1 + *std::max_element(t.maxlayers.begin(), t.maxlayers.end());
    T.e_off = (long long)s->h_energies.size();
    for (int i = 0; i < ne; i++) s->h_energies.push_back(split_pair(energies[i]));
    T.row_off = (long long)s->h_row_off.size();
    const int base = (int)s->h_seg_len.size();
    for (int v : t.offset) s->h_row_off.push_back(base + v);
    // (segment l of a row is density class l: build_trajectories numbers them so)
    for (size_t i = 0; i < t.len_km.size(); i++) s->h_seg_len.push_back(split_pair(t.len_km[i]));
    T.cls_off = (long long)s->h_cls_rho.size();
    s->h_cls_rho.push_back(split_pair(0.0));
    for (int c = 1; c < T.ncls; c++)
        s->h_cls_rho.push_back(split_pair(s->model.rho[c - 1] * s->model.ye[c - 1]));
    T.tab_floats = (size_t)T.ncls * T.ne_pad * kMixFields;  // multiple of kUnit (ne_pad % 32 == 0)
    T.out_floats = ((size_t)9 * nc * ne + kUnit - 1) / kUnit * kUnit;
    T.bins = (long long)nc * ne;
    s->tmpls.push_back(T);
    if (grid) *grid = (int)s->tmpls.size() - 1;
    return CP3_OK;
}

int cp3_server_add_beam_grid(cp3_server* s, const double* energies, int ne, double rho,
                             const double* path_km, int n_baselines, int* grid) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (s->started) return sfail(s, CP3_ERR_UNSUPPORTED, "the server is running");
    if (ne < 1 || !energies || n_baselines < 1 || !path_km) return sfail(s, CP3_ERR_BAD_SIZE, "empty grid");
    Template T;
    T.kind = 1;
    T.ne = ne;
    T.ne_pad = pad_energies(ne);
    T.nrows = n_baselines;
    T.e_off = (long long)s->h_energies.size();
    for (int i = 0; i < ne; i++) s->h_energies.push_back(split_pair(energies[i]));
    T.row_off = (long long)s->h_baselines.size();
    for (int j = 0; j < n_baselines; j++) s->h_baselines.push_back(split_pair(path_km[j]));
    const float2 r = split_pair(rho * kDensityConvert);
    T.rho_e[0] = r.x;
    T.rho_e[1] = r.y;
    T.tab_floats = 0;
    T.out_floats = ((size_t)9 * n_baselines * ne + kUnit - 1) / kUnit * kUnit;
    T.bins = (long long)n_baselines * ne;
    s->tmpls.push_back(T);
    if (grid) *grid = (int)s->tmpls.size() - 1;
    return CP3_OK;
}

int cp3_server_start(cp3_server* s) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (s->started) return CP3_OK;
    if (s->tmpls.empty()) return sfail(s, CP3_ERR_NOT_SET, "no grids registered");
    S_CUDA(s, cudaSetDevice(s->device), "cudaSetDevice");
    S_CUDA(s, upload(s->d_energies, s->h_energies), "upload grids");
    S_CUDA(s, upload(s->d_cls_rho, s->h_cls_rho), "upload grids");
    S_CUDA(s, upload(s->d_row_off, s->h_row_off), "upload grids");
    S_CUDA(s, upload(s->d_seg_len, s->h_seg_len), "upload grids");
    S_CUDA(s, upload(s->d_baselines, s->h_baselines), "upload grids");
    const size_t units = s->pool_bytes / (kUnit * sizeof(float));
    S_CUDA(s, s->d_pool.alloc(units * kUnit), "allocate pool");
    s->pool.init(units);
    for (const Template& T : s->tmpls)
        if ((T.tab_floats + T.out_floats) / kUnit > units)
            return sfail(s, CP3_ERR_BAD_SIZE, "a registered grid does not fit in the pool");
    for (Slot& sl : s->slots)
        if (int rc = capture_slot(s, sl)) return rc;
    s->queues.assign(s->tmpls.size(), {});
    s->by_size.resize(s->tmpls.size());
    for (size_t g = 0; g < s->tmpls.size(); g++) s->by_size[g] = (int)g;
    std::stable_sort(s->by_size.begin(), s->by_size.end(),
                     [&](int a, int b) { return s->tmpls[a].bins < s->tmpls[b].bins; });
    s->started = true;
    s->loop = std::thread(scheduler, s);
    return CP3_OK;
}

int cp3_server_submit(cp3_server* s, int grid, double t12, double t13, double t23, double dcp,
                      int knutype, double dm12sq, double dm23sq, int neutrino_type,
                      unsigned long long* id) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (!s->started) return sfail(s, CP3_ERR_NOT_SET, "cp3_server_start first");
    if (grid < 0 || grid >= (int)s->tmpls.size()) return sfail(s, CP3_ERR_INDEX, "no such grid");
    if (neutrino_type != CP3_NEUTRINO && neutrino_type != CP3_ANTINEUTRINO)
        return sfail(s, CP3_ERR_BAD_ARGUMENT, "neutrino type must be Neutrino or Antineutrino");
    auto r = std::make_shared<Request>();
    r->tmpl = grid;
    MixingInput m;
    m.theta12 = t12;
    m.theta13 = t13;
    m.theta23 = t23;
    m.dcp = dcp;
    m.knutype = knutype;
    m.dm12sq = dm12sq;
    m.dm23sq = dm23sq;
    build_osc_params(m, neutrino_type, &r->params);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->t_submit = now_ns();
        s->requests[r->id] = r;
        s->queues[grid].push_back(r);
        s->queued++;
    }
    s->cv.notify_all();
    if (id) *id = r->id;
    return CP3_OK;
}

int cp3_server_wait(cp3_server* s, unsigned long long id, double timeout_s, int* done) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return sfail(s, CP3_ERR_INDEX, "no such request");
    std::shared_ptr<Request> r = it->second;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(timeout_s));
    // short timed waits: the completion callback notifies without taking the mutex
    while (r->state.load() != kDone && Clock::now() < deadline)
        s->cv.wait_for(lk, std::chrono::microseconds(100));
    const bool finished = r->state.load() == kDone;
    if (done) *done = finished ? 1 : 0;
    if (finished) {
        if (const int st = r->status.load())
            return sfail(s, CP3_ERR_CUDA, st == kReqLaunchFailed ? s->launch_error : std::string(status_text(st)));
    }
    return CP3_OK;
}

int cp3_server_result(cp3_server* s, unsigned long long id, const float** ptr, size_t* count,
                      double* latency_ms) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return sfail(s, CP3_ERR_INDEX, "no such request");
    const Request& r = *it->second;
    if (r.state.load() != kDone) return sfail(s, CP3_ERR_NOT_SET, "request not done");
    if (const int st = r.status.load())
        return sfail(s, CP3_ERR_CUDA, std::string("no result: ") +
                                          (st == kReqLaunchFailed ? s->launch_error : std::string(status_text(st))));
    const Template& T = s->tmpls[r.tmpl];
    if (ptr) *ptr = s->d_pool.ptr + r.pool_off * kUnit + T.tab_floats;
    if (count) *count = (size_t)9 * T.nrows * T.ne;
    if (latency_ms) *latency_ms = (r.t_done - r.t_submit) * 1e-6;
    return CP3_OK;
}

int cp3_server_copy_result(cp3_server* s, unsigned long long id, void* dst) {
    const float* src = nullptr;
    size_t n = 0;
    if (int rc = cp3_server_result(s, id, &src, &n, nullptr)) return rc;
    if (!dst) return sfail(s, CP3_ERR_BAD_ARGUMENT, "null destination");
    S_CUDA(s, cudaSetDevice(s->device), "cudaSetDevice");
    S_CUDA(s, cudaMemcpy(dst, src, n * sizeof(float), cudaMemcpyDeviceToHost), "copy result");
    return CP3_OK;
}

int cp3_server_release(cp3_server* s, unsigned long long id) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->requests.find(id);
        if (it == s->requests.end()) return sfail(s, CP3_ERR_INDEX, "no such request");
        if (it->second->state.load() != kDone) return sfail(s, CP3_ERR_NOT_SET, "request not done");
        s->pool.release(it->second->pool_off, it->second->pool_units);
        s->requests.erase(it);
    }
    s->cv.notify_all();
    return CP3_OK;
}

int cp3_server_poll(cp3_server* s, unsigned long long* ids, int max_ids, double timeout_s, int* n) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (!n || max_ids < 0 || (max_ids > 0 && !ids)) return sfail(s, CP3_ERR_BAD_ARGUMENT, "poll: null output or negative size");
    *n = 0;
    s->record_completions.store(true);
    if (max_ids == 0) return CP3_OK;
    std::unique_lock<std::mutex> lk(s->cq_mu);
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(std::max(timeout_s, 0.0)));
    // timed waits: finish_requests notifies after dropping cq_mu
    while (s->completions.empty() && Clock::now() < deadline)
        s->cq_cv.wait_until(lk, std::min(deadline, Clock::now() + std::chrono::microseconds(200)));
    while (*n < max_ids && !s->completions.empty()) {
        ids[(*n)++] = s->completions.front();
        s->completions.pop_front();
    }
    return CP3_OK;
}

int cp3_server_debug_fail_launches(cp3_server* s, int count) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    if (count < 0) return sfail(s, CP3_ERR_BAD_ARGUMENT, "count must be >= 0");
    std::lock_guard<std::mutex> lk(s->mu);
    s->debug_fail_launches = count;
    return CP3_OK;
}

int cp3_server_stats(cp3_server* s, long long* launches, long long* completed, long long* queued) {
    if (!s) return sfail(nullptr, CP3_ERR_BAD_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (launches) *launches = s->launches.load();
    if (completed) *completed = s->completed.load();
    if (queued) *queued = s->queued;
    return CP3_OK;
}

}  // extern "C"

// cp3_noalloc.cu -- atmospheric mixed-precision propagation without any allocation.
//
// Some callers cannot allocate device memory at the moment they propagate: a fitter that
// owns every byte of the GPU through its own pool, code running inside a region where
// cudaMalloc is forbidden or would synchronise, or a host that must not touch the
// allocator during an MCMC step.  cp3_atmos_mixed_noalloc serves them: it runs the same
// two kernels as a MIXED atmospheric handle (eigen table, then the per-bin kernel), but the
// eigen table and the staged trajectory table live in one file-scope device array whose
// size is fixed when the library is loaded.  Inputs and outputs still belong to the caller.
//
// The first call on each device is its set-up: with that device current it looks up the
// array's device address (cudaGetSymbolAddress) and loads the kernels the call launches.
// Under lazy module loading (the CUDA default) those loads are where the driver places the
// array and the kernels' code in device memory, so the set-up call may allocate; every later
// call on that device allocates nothing.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/cudaprob3_gb300.h"
#include "cp3_host.hpp"
#include "cp3_kernels.hpp"

namespace cp3 {

constexpr size_t kNoAllocScratchFloats = CP3_NOALLOC_SCRATCH_BYTES / sizeof(float);

// The scratch shared by every call on a device.  Every GPU that loads the library holds it
// until the process exits.  Its host-side name is only a stand-in: host code passes the
// address obtained from cudaGetSymbolAddress, never this name.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

namespace {

constexpr size_t kScratchFloats = CP3_NOALLOC_SCRATCH_BYTES / sizeof(float);
constexpr size_t kAlignFloats = 64;  // 256-byte sections
constexpr int kMaxDevices = 64;

std::mutex g_setup_mutex;
float* g_scratch_on[kMaxDevices] = {};

size_t section(size_t floats) { return (floats + kAlignFloats - 1) / kAlignFloats * kAlignFloats; }

int report(char* err, size_t err_len, int code, const char* fmt, long long a = 0, long long b = 0) {
    if (err && err_len > 0) std::snprintf(err, err_len, fmt, a, b);
    return code;
}

__global__ void split_lengths_kernel(const double* __restrict__ len, int n, float2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hi = (float)len[i];
    out[i] = make_float2(hi, (float)(len[i] - (double)hi));
}

// Set-up on the current device: the scratch's device address, and every kernel of the call
// loaded now rather than at its first launch.
cudaError_t setup_device(float** scratch) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    cudaFuncAttributes a;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, split_lengths_kernel);
    if (e == cudaSuccess) e = preload_table_mixed();
    if (e == cudaSuccess) e = preload_atmos_mixed();
    if (e == cudaSuccess) *scratch = static_cast<float*>(p);
    return e;
}

}  // namespace
}  // namespace cp3

using namespace cp3;

extern "C" int cp3_atmos_mixed_noalloc(int device, const double* d_energies, int n_energies,
                                       const int* seg_offset, const double* seg_len_km,
                                       const int* seg_class, int n_cosines,
                                       const double* class_rho_e, int n_classes, double theta12,
                                       double theta13, double theta23, double dcp, int knutype,
                                       double dm12sq, double dm23sq, int neutrino_type,
                                       float* d_out, void* stream, char* err, size_t err_len) {
    if (err && err_len > 0) err[0] = '\0';
    // ---- arguments, on the host ---------------------------------------------------------
    if (!d_energies || !seg_offset || !seg_len_km || !seg_class || !class_rho_e || !d_out)
        return report(err, err_len, CP3_ERR_BAD_ARGUMENT, "null input or output pointer");
    if (n_energies < 1 || n_cosines < 1 || n_classes < 1)
        return report(err, err_len, CP3_ERR_BAD_SIZE,
                      "n_energies, n_cosines and n_classes must be positive");
    if (neutrino_type != CP3_NEUTRINO && neutrino_type != CP3_ANTINEUTRINO)
        return report(err, err_len, CP3_ERR_BAD_ARGUMENT, "neutrino type must be 0 or 1");
    if (seg_offset[0] != 0)
        return report(err, err_len, CP3_ERR_BAD_ARGUMENT, "seg_offset[0] must be 0");
    for (int ic = 0; ic < n_cosines; ic++) {
        const int len = seg_offset[ic + 1] - seg_offset[ic];
        if (len < 1 || len > kMaxSegments)
            return report(err, err_len, CP3_ERR_LAYER_LIMIT,
                          "cosine row %lld has %lld segments (1..129 allowed)", ic, len);
    }
    const int n_seg = seg_offset[n_cosines];
    // The kernels read the table of class l for a row's segment l (the numbering of
    // cp3_trajectory_table): any other class array is refused rather than ignored.
    for (int ic = 0; ic < n_cosines; ic++)
        for (int s = seg_offset[ic]; s < seg_offset[ic + 1]; s++) {
            const int l = s - seg_offset[ic];
            if (seg_class[s] != l || l >= n_classes)
                return report(err, err_len, CP3_ERR_BAD_ARGUMENT,
                              "segment %lld has class %lld: segment l of a row must be class l "
                              "< n_classes (cp3_trajectory_table's numbering)",
                              s, seg_class[s]);
        }

    // ---- scratch plan: [offsets][lengths f64][lengths f32 pair][class rho][table] ---------
    const size_t ne_pad = (size_t)pad_energies(n_energies);
    const size_t off_f = 0;
    const size_t lend_f = off_f + section((size_t)n_cosines + 1);
    const size_t lenf_f = lend_f + section(2 * (size_t)n_seg);
    const size_t rho_f = lenf_f + section(2 * (size_t)n_seg);
    const size_t tab_f = rho_f + section(2 * (size_t)n_classes);
    const size_t need = tab_f + (size_t)n_classes * kMixFields * ne_pad;
    if (need > kScratchFloats)
        return report(err, err_len, CP3_ERR_BAD_SIZE,
                      "this grid needs %lld bytes of scratch; the no-allocation scratch holds %lld "
                      "bytes (fewer energies, cosines or shells fit)",
                      (long long)(need * sizeof(float)), (long long)CP3_NOALLOC_SCRATCH_BYTES);

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev ||
        device >= kMaxDevices) {
        cudaGetLastError();
        return report(err, err_len, CP3_ERR_BAD_ARGUMENT, "device %lld is not available", device);
    }
    int prev = -1;
    cudaGetDevice(&prev);

    // ---- once per device, with that device current: the scratch's device address and the
    //      kernels loaded (the set-up call) ------------------------------------------------
    float* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_on[device]) {
            cudaError_t e = cudaSetDevice(device);
            float* p = nullptr;
            if (e == cudaSuccess) e = setup_device(&p);
            if (e != cudaSuccess) {
                cudaGetLastError();
                if (prev >= 0) cudaSetDevice(prev);
                if (err && err_len > 0)
                    std::snprintf(err, err_len, "no-allocation set-up: %s", cudaGetErrorString(e));
                return CP3_ERR_CUDA;
            }
            g_scratch_on[device] = p;
        }
        base = g_scratch_on[device];
    }

    cudaError_t e = cudaSetDevice(device);
    const cudaStream_t s = (cudaStream_t)stream;
    int* d_off = reinterpret_cast<int*>(base + off_f);
    double* d_len = reinterpret_cast<double*>(base + lend_f);
    float2* d_len2 = reinterpret_cast<float2*>(base + lenf_f);
    double* d_rho = reinterpret_cast<double*>(base + rho_f);
    float* d_tab = base + tab_f;
    // Host arrays are staged by cudaMemcpyAsync; from pageable memory the copy has taken the
    // data when the call returns, so the caller may reuse its arrays at once.  Nothing in
    // the scratch needs clearing: each call writes every element it later reads.
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, seg_offset, sizeof(int) * (n_cosines + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_len, seg_len_km, sizeof(double) * n_seg, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_rho, class_rho_e, sizeof(double) * n_classes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        split_lengths_kernel<<<(n_seg + 255) / 256, 256, 0, s>>>(d_len, n_seg, d_len2);
        e = cudaGetLastError();
    }
    OscParams p;
    MixingInput m;
    m.theta12 = theta12;
    m.theta13 = theta13;
    m.theta23 = theta23;
    m.dcp = dcp;
    m.knutype = knutype;
    m.dm12sq = dm12sq;
    m.dm23sq = dm23sq;
    build_osc_params(m, neutrino_type == CP3_ANTINEUTRINO, &p);
    if (e == cudaSuccess) e = launch_table_mixed(p, d_energies, n_energies, d_rho, n_classes, d_tab, s);
    if (e == cudaSuccess)
        e = launch_atmos_mixed(p, d_tab, n_energies, d_off, d_len2, n_cosines, d_out, s);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (err && err_len > 0) std::snprintf(err, err_len, "CUDA: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? CP3_ERR_OOM : CP3_ERR_CUDA;
    }
    return CP3_OK;
}

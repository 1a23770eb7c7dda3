// cp3_peaks.cu -- scalar FMA throughput of the device (bench support, libcp3peaks.so).
//
// The roofline denominators of the propagation kernels are the FP32 and FP64 scalar pipes,
// which the pool's measured-peaks file (an HBM copy and a bf16 GEMM) does not cover.  This
// kernel measures them live, under the same clocks as the bench: every thread runs eight
// independent dependent FMA chains (enough to cover the pipe latency), and the device time
// of a launch that fills every SM several times over gives FLOP/s = 2 x FMAs / time.
// A third variant runs the chains on float pairs with the paired FP32 FMA of sm_100+
// (__ffma2_rn, two FMAs per instruction), the FP32 pipe's throughput when instruction issue
// is not the limit.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) fma_chains(T* out, int iters, T b, T c) {
    T a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k];
    if (s == (T)-12345.0) out[blockIdx.x * kThreads + threadIdx.x] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(kThreads) fma2_chains(float* out, int iters, float b, float c) {
    float2 a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++)
        a[k] = make_float2((float)(threadIdx.x + k) * 1e-3f, (float)(threadIdx.x + k + 1) * 1e-3f);
    const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) a[k] = __ffma2_rn(a[k], b2, c2);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k].x + a[k].y;
    if (s == -12345.0f) out[blockIdx.x * kThreads + threadIdx.x] = s;
}

template <typename T>
void launch_chains(bool paired, int blocks, T* out, int iters, T b, T c, cudaStream_t s) {
    fma_chains<T><<<blocks, kThreads, 0, s>>>(out, iters, b, c);
}
template <>
void launch_chains<float>(bool paired, int blocks, float* out, int iters, float b, float c,
                          cudaStream_t s) {
    if (paired)
        fma2_chains<<<blocks, kThreads, 0, s>>>(out, iters, b, c);
    else
        fma_chains<float><<<blocks, kThreads, 0, s>>>(out, iters, b, c);
}

template <typename T>
int run(int device, int iters, bool paired, double* tflops, double* ms_out) {
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * kThreads) != cudaSuccess) return 2;
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const T b = (T)0.999999, c = (T)1e-7;
    for (int w = 0; w < 3; w++) launch_chains<T>(paired, blocks, out, iters, b, c, s);
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0, s);
        launch_chains<T>(paired, blocks, out, iters, b, c, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const int err = cudaGetLastError() != cudaSuccess ? 3 : 0;
    const double flops = (paired ? 4.0 : 2.0) * kChains * (double)iters * blocks * kThreads;
    *tflops = flops / (best * 1e-3) / 1e12;
    *ms_out = best;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    return err;
}

}  // namespace

// mode 0: FP32 FMA, 1: FP64 FMA, 2: paired FP32 FMA (__ffma2_rn).
extern "C" int cp3peaks_fma_tflops(int mode, int device, int iters, double* tflops, double* ms) {
    if (mode == 1) return run<double>(device, iters, false, tflops, ms);
    return run<float>(device, iters, mode == 2, tflops, ms);
}

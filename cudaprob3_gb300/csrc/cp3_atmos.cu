// cp3_atmos.cu -- per-bin kernels: atmospheric FP64 and mixed, beam mixed.
//
// Mapping: one CTA = one cosine row x a tile of consecutive energies (kBlock, or kBlockMixed
// for the mixed table kernel), one thread = one (cosine, energy) bin.  The row's trajectory
// (its segment lengths, a few hundred bytes; segment l reads density class l) is staged in
// shared memory; every thread of the CTA then walks the same segment list, so control flow
// is uniform.  The per-(class, energy) eigen tables are read contiguously across a warp
// (one entry per energy) and stay L2-resident.  The result
// [9][n_cosines][n_energies] is written one channel plane at a time: each warp store is
// 32 consecutive elements (128 B in FP32, 256 B in FP64).
#include "cp3_device.cuh"
#include "cp3_kernels.hpp"
#include "cp3_f64.cuh"
#include "cp3_mixed.cuh"

namespace cp3 {

namespace {

constexpr int kBlock = 128;
// The mixed table kernel's CTA: one row x 256 energies (1 % faster than 128 on the 59-shell
// grid: half the trajectory staging per bin; 64 was 1 % slower).
constexpr int kBlockMixed = 256;
constexpr int kMaxGridY = 65535;

// ------------------------------------------------------------------------------------
// FP64: physics::calculate_atmos (physics.hpp:789-1150), within 1e-12 of the reference.
//
// The same physics as the reference in the rotated real basis of the mixed kernels
// (cp3_mixed.cuh), in double precision: every layer is S = sum_k e^{i arg_k} P_k with the
// reference's own phases arg_k = -2.534 dmMatVac[k][0] L / E (getArg, physics.hpp:439-450)
// and the rotated-basis projectors P_k = u_k u_k^T; dropping the global phase e^{i arg_0},
//   S ~ 1 + z1 u1 u1^T + z2 u2 u2^T,  z_k = e^{i arg_k} conj(e^{i arg_0}) - 1,
// applied as two rank-1 updates, and the palindrome (physics.hpp:956-990) as
// W (B^T S_M B) S_0 W^+ with B = S_{M-1}..S_1: M+1 layer applications instead of 2M-1
// complex 3x3 products.  The phases are formed exactly as the reference forms them, so
// their roundings -- which matter over ~120 layers of up to ~800 rad -- are the reference's.

// Table entry (10 doubles, five 16-byte words): u1, u2, dmMatVac[0..2][0], 1 unused.
__device__ __forceinline__ void layer64_from_table(const double* __restrict__ t, double L,
                                                   double E, double rE, Layer64& f,
                                                   double arg[3]) {
    const double2* t2 = reinterpret_cast<const double2*>(t);
    const double2 a = __ldg(t2), b = __ldg(t2 + 1), c = __ldg(t2 + 2), d = __ldg(t2 + 3),
                  e = __ldg(t2 + 4);
    f.u[0][0] = a.x;
    f.u[0][1] = a.y;
    f.u[0][2] = b.x;
    f.u[1][0] = b.y;
    f.u[1][1] = c.x;
    f.u[1][2] = c.y;
    const double dmv[3] = {d.x, d.y, e.x};
    layer64_phases(dmv, L, E, rE, f, arg);
}

// G <- S G
__device__ __forceinline__ void apply_left64(const Layer64& f, cm3& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const double* u = f.u[k];
        const cd z = f.z[k];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const double wr = u[0] * G.a[0][j].re + u[1] * G.a[1][j].re + u[2] * G.a[2][j].re;
            const double wi = u[0] * G.a[0][j].im + u[1] * G.a[1][j].im + u[2] * G.a[2][j].im;
            const double yr = z.re * wr - z.im * wi, yi = z.re * wi + z.im * wr;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                G.a[i][j].re += u[i] * yr;
                G.a[i][j].im += u[i] * yi;
            }
        }
    }
}

// G <- G S
__device__ __forceinline__ void apply_right64(const Layer64& f, cm3& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const double* u = f.u[k];
        const cd z = f.z[k];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const double wr = G.a[i][0].re * u[0] + G.a[i][1].re * u[1] + G.a[i][2].re * u[2];
            const double wi = G.a[i][0].im * u[0] + G.a[i][1].im * u[1] + G.a[i][2].im * u[2];
            const double yr = wr * z.re - wi * z.im, yi = wr * z.im + wi * z.re;
#pragma unroll
            for (int j = 0; j < 3; j++) {
                G.a[i][j].re += yr * u[j];
                G.a[i][j].im += yi * u[j];
            }
        }
    }
}

// Production-height averaging (physics.hpp:997-1067), the reference's shift factors for the
// pairs (k, q) = (1,0), (2,0), (2,1) and each initial flavour f: sf[pair][f] = sum over bins
// of prob * sinc(d hw / 2) e^{i d hm}, d = darg0[k] - darg0[q]; the diagonal is 1.
struct WParams64 {
    double w[4];  // c23, s23, cos d, sin d
};

struct AvgInput {
    const double* prob;    // [2][3][ne][nc][nb]
    const double* shift;   // [nc][nb + 1] path-length shifts at the bin edges, cm
    const double* air_cm;  // [nc] segment 0 length, cm
    int nb, type;
};

// math::defined_sinc (math.hpp:49-55) as the reference evaluates it: its unqualified abs()
// binds to int abs(int), so the series branch runs for every |x| < 1.
__device__ __forceinline__ double sinc_reference(double x) {
    if (fabs(x) >= 1.0) return sin(x) / x;
    return 1.0 - x * x / 6. + x * x * x * x / 120.;
}

__device__ __forceinline__ void avg_shift_factors(const AvgInput& av, int ic, int nc, int ie, int ne,
                                                  const double arg0[3], cd sf[3][3]) {
    const double dist = av.air_cm[ic];
    double d0[3];
#pragma unroll
    for (int k = 0; k < 3; k++) d0[k] = dist == 0. ? 0. : arg0[k] / dist;
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int f = 0; f < 3; f++) sf[q][f] = cd{0.0, 0.0};
    const int pa[3] = {1, 2, 2}, pb[3] = {0, 0, 1};
    const double* sh = av.shift + (size_t)ic * (av.nb + 1);
    for (int p = 0; p < av.nb; p++) {
        const double h0 = sh[p], h1 = sh[p + 1];
        const double hm = (h1 + h0) / 2., hw = (h1 - h0);
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const double d = d0[pa[q]] - d0[pb[q]];
            const double sarg = 0.5 * d * hw;
            const double fre = sinc_reference(sarg) * cos(d * hm);
            const double fim = sinc_reference(sarg) * sin(d * hm);
#pragma unroll
            for (int f = 0; f < 3; f++) {
                const size_t idx = (((size_t)(av.type * 3 + f) * ne + ie) * nc + ic) * av.nb + p;
                const double w = av.prob[idx];
                sf[q][f].re += w * fre;
                sf[q][f].im += w * fim;
            }
        }
    }
}

// With production-height averaging, the reference's probability (physics.hpp:1102-1130):
// the amplitude split over the air layer's eigencomponents, Product_k = fin C_atm[k] =
// W G P_k e_k W^+ (e_0 = 1 once the global phase is dropped), |Product_k|^2 summed and the
// cross terms weighted by the shift factors sf.  The eigen labels are the reference's (the
// FP64 layer data keep its mass order), so each pair (k, q) meets its own shift factor.
// Out of line: it is the rare path and keeps its registers out of the common one.
__device__ __noinline__ void finish_averaged64(const cm3& G, const Layer64& F0, const double* w,
                                               const cd (*sf)[3], double* __restrict__ out,
                                               size_t plane) {
    cm3 Prod[3];
    cm3 Y0 = G;
#pragma unroll
    for (int kk = 0; kk < 2; kk++) {
        const double* u = F0.u[kk];
        const cd e{1.0 + F0.z[kk].re, F0.z[kk].im};
        cm3 Y;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const cd gu{G.a[i][0].re * u[0] + G.a[i][1].re * u[1] + G.a[i][2].re * u[2],
                        G.a[i][0].im * u[0] + G.a[i][1].im * u[1] + G.a[i][2].im * u[2]};
            const cd ge{gu.re * e.re - gu.im * e.im, gu.re * e.im + gu.im * e.re};
#pragma unroll
            for (int j = 0; j < 3; j++) {
                Y.a[i][j] = cd{ge.re * u[j], ge.im * u[j]};
                Y0.a[i][j].re -= gu.re * u[j];
                Y0.a[i][j].im -= gu.im * u[j];
            }
        }
        to_flavour64(Y, w, Prod[kk + 1]);
    }
    to_flavour64(Y0, w, Prod[0]);
    const int pair[3][3] = {{-1, -1, -1}, {0, -1, -1}, {1, 2, -1}};  // (k, q) -> index, q < k
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double prob = 0.0;
            for (int k = 0; k < 3; k++) {
                const cd Pk = Prod[k].a[i][j];
                prob += Pk.re * Pk.re + Pk.im * Pk.im;
                for (int q = 0; q < k; q++) {
                    const cd Pq = Prod[q].a[i][j];
                    const cd t = sf[pair[k][q]][j];
                    prob += 2. * Pq.re * Pk.re * t.re + 2. * Pq.im * Pk.im * t.re +
                            2. * Pq.im * Pk.re * t.im - 2. * Pq.re * Pk.im * t.im;
                }
            }
            // Prob[i][j] (i final, j initial) is P(j -> i): channel j*3+i.
            out[(size_t)(j * 3 + i) * plane] = prob;
        }
}

// One FP64 bin over M+1 layers; seg(l, F, arg) fills layer l (0 = air) and its phases.
template <class SegFn>
__device__ __forceinline__ void atmos_bin_f64(SegFn seg, int M, const double* w,
                                              const AvgInput& av, int ic, int nc, int ie, int ne,
                                              double* __restrict__ out, size_t plane) {
    cm3 G;
    Layer64 F;
    double arg[3];
    if (M == 0) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) G.a[i][j] = cd{i == j ? 1.0 : 0.0, 0.0};
    } else {
        seg(1, F, arg);
        layer_to_gen64(F, G);  // B = S_1
        if (M > 1) {
            for (int l = 2; l < M; l++) {
                seg(l, F, arg);
                apply_left64(F, G);
            }
            seg(M, F, arg);
            cm3 X = G;
            apply_left64(F, X);  // X = S_M B
            cm3 Q;               // Q = B^T X (symmetric)
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = i; j < 3; j++) {
                    double re = 0.0, im = 0.0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const cd b = G.a[k][i], x = X.a[k][j];
                        re += b.re * x.re - b.im * x.im;
                        im += b.re * x.im + b.im * x.re;
                    }
                    Q.a[i][j] = cd{re, im};
                    Q.a[j][i] = cd{re, im};
                }
            G = Q;
        }
    }
    seg(0, F, arg);  // the air layer, applied last: A2 = G S_0
    if (M == 0 && av.nb == 0) {  // the air layer alone: the one-layer expansion
        layer_store64(layer_coefficients64(F.u, w), F.z, out, plane);
        return;
    }
    if (av.nb > 0) {
        cd sf[3][3];
        avg_shift_factors(av, ic, nc, ie, ne, arg, sf);
        finish_averaged64(G, F, w, sf, out, plane);
        return;
    }
    apply_right64(F, G);
    cm3 A;
    to_flavour64(G, w, A);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            out[(size_t)(j * 3 + i) * plane] = A.a[i][j].re * A.a[i][j].re + A.a[i][j].im * A.a[i][j].im;
}

// FP64 atmospheric bins, quadratic density: every segment carries its own density, so its
// eigen-system is solved per segment (the reference's getMfast, then the rotated projectors).
__global__ void __launch_bounds__(kBlock)
    atmos_f64_inline_kernel(const __grid_constant__ OscParams p, const double* __restrict__ energies,
                            int ne, const int* __restrict__ seg_off,
                            const double* __restrict__ seg_len, const double* __restrict__ seg_rho,
                            int ic0, int nc, AvgInput av, double* __restrict__ out) {
    __shared__ double s_len[kMaxSegments];
    __shared__ double s_rho[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) {
        s_len[i] = seg_len[s0 + i];
        s_rho[i] = seg_rho[s0 + i];
    }
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie], rE = 1.0 / E;
    atmos_bin_f64(
        [&](int l, Layer64& F, double arg[3]) {
            double dmv[3];
            rotated_layer_f64(&p, E, s_rho[l], F.u, dmv);
            layer64_phases(dmv, s_len[l], E, rE, F, arg);
        },
        nseg - 1, p.w, av, ic, nc, ie, ne, out + (size_t)ic * ne + ie, (size_t)nc * ne);
}

__global__ void __launch_bounds__(kBlock)
    atmos_f64_kernel(const double* __restrict__ energies, int ne, int ne_pad,
                     const double* __restrict__ table, const int* __restrict__ seg_off,
                     const double* __restrict__ seg_len, int ic0, int nc,
                     const __grid_constant__ WParams64 w, AvgInput av, double* __restrict__ out) {
    __shared__ double s_len[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) s_len[i] = seg_len[s0 + i];
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie], rE = 1.0 / E;
    const size_t cls_stride = (size_t)kF64Fields * ne_pad;
    const double* tab = table + (size_t)ie * kF64Fields;
    atmos_bin_f64(
        [&](int l, Layer64& F, double arg[3]) {
            layer64_from_table(tab + l * cls_stride, s_len[l], E, rE, F, arg);  // class l
        },
        nseg - 1, w.w, av, ic, nc, ie, ne, out + (size_t)ic * ne + ie, (size_t)nc * ne);
}

// Mixed atmospheric bins (the physics of calculate_atmos rearranged for FP32: see
// cp3_mixed.cuh).
__global__ void __launch_bounds__(kBlockMixed)
    atmos_mixed_kernel(WParams w, const float* __restrict__ table, int ne, int ne_pad,
                       const int* __restrict__ seg_off, const float2* __restrict__ seg_len,
                       int ic0, int nc, float* __restrict__ out) {
    __shared__ float2 s_len[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlockMixed) s_len[i] = seg_len[s0 + i];
    __syncthreads();
    const int ie = blockIdx.x * kBlockMixed + threadIdx.x;
    if (ie >= ne) return;
    atmos_bin_mixed(table + (size_t)ie * kMixFields, (size_t)kMixFields * ne_pad, s_len, nseg - 1,
                    w, out + (size_t)ic * ne + ie, (size_t)nc * ne);
}

// Mixed atmospheric bins, quadratic density: every segment solves its own eigen-system.
__global__ void __launch_bounds__(kBlock)
    atmos_mixed_inline_kernel(const __grid_constant__ OscParams p, WParams w,
                              const double* __restrict__ energies, int ne,
                              const int* __restrict__ seg_off, const float2* __restrict__ seg_len,
                              const double* __restrict__ seg_rho, int ic0, int nc,
                              float* __restrict__ out) {
    __shared__ float2 s_len[kMaxSegments];
    __shared__ double s_rho[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) {
        s_len[i] = seg_len[s0 + i];
        s_rho[i] = seg_rho[s0 + i];
    }
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie];
    atmos_bin_mixed_with([&](int l, Layer& F) { segment_layer_inline(&p, E, s_rho[l], s_len[l], F); },
                         nseg - 1, w, out + (size_t)ic * ne + ie, (size_t)nc * ne);
}

// Beam, mixed: per-bin eigen-decomposition with double-float refinement
// (rotated_eigen_mixed), double-float phase, FP32 matrix work.
__global__ void __launch_bounds__(kBlock)
    beam_mixed_kernel(const __grid_constant__ OscParams p, WParams w,
                      const float2* __restrict__ energies, int ne, float2 rho_e, float2 L,
                      float* __restrict__ out) {
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    beam_bin_mixed(&p, w, to_df(energies[ie]), to_df(rho_e), &L, 1, out + ie, (size_t)ne, 0);
}

}  // namespace

cudaError_t launch_atmos_f64(const OscParams& p, const double* energies, int ne,
                             const double* table, const int* seg_off, const double* seg_len,
                             int n_cosines, const AvgArrays& avg, double* out,
                             cudaStream_t s, RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const int ne_pad = pad_energies(ne);
    const AvgInput av{avg.prob, avg.shift, avg.air_cm, avg.n_bins, p.anti};
    const WParams64 w{{p.w[0], p.w[1], p.w[2], p.w[3]}};
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        atmos_f64_kernel<<<grid, kBlock, 0, s>>>(energies, ne, ne_pad, table, seg_off, seg_len,
                                                 ic0, n_cosines, w, av, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_atmos_mixed(const OscParams& p, const float* table, int ne,
                               const int* seg_off, const float2* seg_len, int n_cosines,
                               float* out, cudaStream_t s, RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const int ne_pad = pad_energies(ne);
    const WParams w = wparams(p);
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlockMixed - 1) / kBlockMixed, rows);
        atmos_mixed_kernel<<<grid, kBlockMixed, 0, s>>>(w, table, ne, ne_pad, seg_off, seg_len,
                                                   ic0, n_cosines, out);
    }
    return cudaGetLastError();
}

cudaError_t preload_atmos_mixed() {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, atmos_mixed_kernel);
}

cudaError_t launch_atmos_inline(const OscParams& p, bool mixed, const double* energies, int ne,
                                const int* seg_off, const void* seg_len, const double* seg_rho,
                                int n_cosines, const AvgArrays& avg, void* out, cudaStream_t s,
                                RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const AvgInput av{avg.prob, avg.shift, avg.air_cm, avg.n_bins, p.anti};
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        if (mixed)
            atmos_mixed_inline_kernel<<<grid, kBlock, 0, s>>>(p, wparams(p), energies, ne, seg_off,
                                                              (const float2*)seg_len, seg_rho, ic0,
                                                              n_cosines, (float*)out);
        else
            atmos_f64_inline_kernel<<<grid, kBlock, 0, s>>>(p, energies, ne, seg_off,
                                                            (const double*)seg_len, seg_rho, ic0,
                                                            n_cosines, av, (double*)out);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Mixed atmospheric bins with production-height averaging (physics.hpp:997-1130): the
// amplitude split over the air layer's eigencomponents as in finish_averaged64, in FP32,
// with the shift factors' phases reduced in double-float (d hm reaches hundreds of rad).

__device__ __forceinline__ float sinc_reference_f(float x) {
    // math::defined_sinc (math.hpp:49-55) as the reference evaluates it (int abs: the series
    // branch for every |x| < 1)
    if (fabsf(x) >= 1.0f) return sinf(x) / x;
    return 1.0f - x * x / 6.0f + x * x * x * x / 120.0f;
}

// Flavour-basis amplitude A = W A2 W^+ in FP32 (the transform of store_probabilities).
__device__ __forceinline__ void to_flavour_f32(const cg9& A2, const WParams& w, cg9& A) {
    cg9 Y;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const cf a1 = A2.a[i][1], a2 = A2.a[i][2];
        const cf f{a2.re * w.er + a2.im * w.ei, a2.im * w.er - a2.re * w.ei};  // e* a2
        Y.a[i][0] = A2.a[i][0];
        Y.a[i][1] = cf{fmaf(w.c, a1.re, w.s * f.re), fmaf(w.c, a1.im, w.s * f.im)};
        Y.a[i][2] = cf{fmaf(-w.s, a1.re, w.c * f.re), fmaf(-w.s, a1.im, w.c * f.im)};
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const cf y1 = Y.a[1][j], y2 = Y.a[2][j];
        const cf g{y2.re * w.er - y2.im * w.ei, y2.re * w.ei + y2.im * w.er};  // e y2
        A.a[0][j] = Y.a[0][j];
        A.a[1][j] = cf{fmaf(w.c, y1.re, w.s * g.re), fmaf(w.c, y1.im, w.s * g.im)};
        A.a[2][j] = cf{fmaf(-w.s, y1.re, w.c * g.re), fmaf(-w.s, y1.im, w.c * g.im)};
    }
}

// One averaged bin: the chain of segments 1..M (seg(l, F) gives segment l's layer), then the
// amplitude split over the air layer's eigencomponents (F0, with phase rates om1, om2 in turns
// per km) and the reference's cross terms with their shift factors.
template <class SegFn>
__device__ __forceinline__ void atmos_bin_mixed_avg(SegFn seg, int M, const Layer& F0, df om1,
                                                    df om2, const WParams& w, const AvgMixed& av,
                                                    int ic, int nc, int ie, int ne,
                                                    float* __restrict__ out) {
    cg9 G;
    if (M == 0) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) G.a[i][j] = cf{i == j ? 1.0f : 0.0f, 0.0f};
    } else {
        chain_mixed(seg, M, G);
        if (M >= kNewtonSchulzMinShells) newton_schulz(G);
    }
    // shift factors of the pairs (1,0), (2,0), (2,1): the reference's d = d0[k] - d0[q] is
    // -(omega_k - omega_q) per km of path-length shift (omega_0 = 0); the rates are in turns
    // per km
    const df dom[3] = {om1, om2, df_sub(om2, om1)};
    cf sf[3][3];
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int f = 0; f < 3; f++) sf[q][f] = cf{0.0f, 0.0f};
    for (int b = 0; b < av.nb; b++) {
        const float2 hm = av.hm[(size_t)ic * av.nb + b];
        const float hw = av.hw[(size_t)ic * av.nb + b];
        float pr[3];
#pragma unroll
        for (int f = 0; f < 3; f++)
            pr[f] = av.prob[((((size_t)av.type * 3 + f) * ne + ie) * nc + ic) * av.nb + b];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float lo;
            const float r = reduced_turn(dom[q].hi, dom[q].lo, -hm.x, -hm.y, lo);  // d hm
            float er, ei;
            unit_turn_minus_one(-r, -lo, er, ei);  // e^{i d hm} - 1
            er += 1.0f;
            const float sc = sinc_reference_f(-kPiF * dom[q].hi * hw);  // d hw / 2 in rad
#pragma unroll
            for (int f = 0; f < 3; f++) {
                sf[q][f].re = fmaf(pr[f] * sc, er, sf[q][f].re);
                sf[q][f].im = fmaf(pr[f] * sc, ei, sf[q][f].im);
            }
        }
    }

    // Product_k = W G P_k e_k W^+, k = 0 (the rest), 1, 2
    cg9 Pr[3], Y0 = G;
#pragma unroll
    for (int kk = 0; kk < 2; kk++) {
        const float* u = F0.u[kk];
        const cf e{1.0f + F0.z[kk][0], F0.z[kk][1]};
        cg9 Y;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const cf gu{fmaf(G.a[i][0].re, u[0], fmaf(G.a[i][1].re, u[1], G.a[i][2].re * u[2])),
                        fmaf(G.a[i][0].im, u[0], fmaf(G.a[i][1].im, u[1], G.a[i][2].im * u[2]))};
            const cf ge = cmulf(gu, e);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                Y.a[i][j] = cf{ge.re * u[j], ge.im * u[j]};
                Y0.a[i][j].re = fmaf(-gu.re, u[j], Y0.a[i][j].re);
                Y0.a[i][j].im = fmaf(-gu.im, u[j], Y0.a[i][j].im);
            }
        }
        to_flavour_f32(Y, w, Pr[kk + 1]);
    }
    to_flavour_f32(Y0, w, Pr[0]);
    const size_t plane = (size_t)nc * ne;
    float* o = out + (size_t)ic * ne + ie;
    const int pair[3][3] = {{-1, -1, -1}, {0, -1, -1}, {1, 2, -1}};  // (k, q) -> index, q < k
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float prob = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const cf Pk = Pr[k].a[i][j];
                prob = fmaf(Pk.re, Pk.re, fmaf(Pk.im, Pk.im, prob));
#pragma unroll
                for (int q = 0; q < k; q++) {
                    const cf Pq = Pr[q].a[i][j], t = sf[pair[k][q]][j];
                    // 2 Re(conj(Pq) Pk t)
                    const float cr = fmaf(Pq.re, Pk.re, Pq.im * Pk.im);
                    const float ci = fmaf(Pq.re, Pk.im, -Pq.im * Pk.re);
                    prob = fmaf(2.0f, fmaf(cr, t.re, -ci * t.im), prob);
                }
            }
            o[(size_t)(j * 3 + i) * plane] = prob;  // Prob[i][j] is P(j -> i): channel j*3+i
        }
}


__global__ void __launch_bounds__(kBlock)
    atmos_mixed_avg_kernel(WParams w, const float* __restrict__ table, int ne, int ne_pad,
                           const int* __restrict__ seg_off, const float2* __restrict__ seg_len,
                           int ic0, int nc, AvgMixed av, float* __restrict__ out) {
    __shared__ float2 s_len[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) s_len[i] = seg_len[s0 + i];
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const float* tab = table + (size_t)ie * kMixFields;
    const size_t cls_stride = (size_t)kMixFields * ne_pad;
    auto seg = [&](int l, Layer& F) { layer_from_table(tab + l * cls_stride, s_len[l], F); };
    Layer F0;
    const float* t0 = tab;  // class 0: the air
    layer_from_table(t0, s_len[0], F0);
    const df om1{__ldg(t0 + 6), __ldg(t0 + 8)}, om2{__ldg(t0 + 7), __ldg(t0 + 9)};
    atmos_bin_mixed_avg(seg, nseg - 1, F0, om1, om2, w, av, ic, nc, ie, ne, out);
}

// The same with the quadratic density model: every segment solves its own eigen-system
// (segment_layer_inline), the air layer's included.
__global__ void __launch_bounds__(kBlock)
    atmos_mixed_inline_avg_kernel(const __grid_constant__ OscParams p, WParams w,
                                  const double* __restrict__ energies, int ne,
                                  const int* __restrict__ seg_off,
                                  const float2* __restrict__ seg_len,
                                  const double* __restrict__ seg_rho, int ic0, int nc,
                                  AvgMixed av, float* __restrict__ out) {
    __shared__ float2 s_len[kMaxSegments];
    __shared__ double s_rho[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) {
        s_len[i] = seg_len[s0 + i];
        s_rho[i] = seg_rho[s0 + i];
    }
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie];
    auto seg = [&](int l, Layer& F) { segment_layer_inline(&p, E, s_rho[l], s_len[l], F); };
    Layer F0;
    float om[2][2];
    segment_layer_inline_rates(&p, E, s_rho[0], s_len[0], F0, om);
    atmos_bin_mixed_avg(seg, nseg - 1, F0, df{om[0][0], om[0][1]}, df{om[1][0], om[1][1]}, w, av,
                        ic, nc, ie, ne, out);
}

cudaError_t launch_atmos_mixed_avg(const OscParams& p, const float* table, int ne,
                                   const int* seg_off, const float2* seg_len, int n_cosines,
                                   const AvgMixed& av, float* out, cudaStream_t s,
                                   RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const int ne_pad = pad_energies(ne);
    const WParams w = wparams(p);
    AvgMixed a = av;
    a.type = p.anti;
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        atmos_mixed_avg_kernel<<<grid, kBlock, 0, s>>>(w, table, ne, ne_pad, seg_off, seg_len,
                                                       ic0, n_cosines, a, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_atmos_mixed_inline_avg(const OscParams& p, const double* energies, int ne,
                                          const int* seg_off, const float2* seg_len,
                                          const double* seg_rho, int n_cosines,
                                          const AvgMixed& av, float* out, cudaStream_t s,
                                          RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const WParams w = wparams(p);
    AvgMixed a = av;
    a.type = p.anti;
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        atmos_mixed_inline_avg_kernel<<<grid, kBlock, 0, s>>>(p, w, energies, ne, seg_off, seg_len,
                                                              seg_rho, ic0, n_cosines, a, out);
    }
    return cudaGetLastError();
}

// One channel plane [nc][ne] of a result, transposed to [ne][nc] doubles (the layout of
// getProbabilityArr, atmoscudapropagator.cu:238-257): 32 x 32 tiles through shared memory,
// coalesced on both sides.
template <class T>
__global__ void __launch_bounds__(32 * 8)
    plane_transpose_kernel(const T* __restrict__ src, int nc, int ne, double* __restrict__ dst) {
    __shared__ double tile[32][33];
    const int e0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int c = c0 + k, e = e0 + threadIdx.x;
        if (c < nc && e < ne) tile[k][threadIdx.x] = (double)src[(size_t)c * ne + e];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int e = e0 + k, c = c0 + threadIdx.x;
        if (c < nc && e < ne) dst[(size_t)e * nc + c] = tile[threadIdx.x][k];
    }
}

cudaError_t launch_plane_transpose(const void* src, bool is_float, int nc, int ne, double* dst,
                                   cudaStream_t s) {
    if (nc <= 0 || ne <= 0) return cudaSuccess;
    const dim3 grid((ne + 31) / 32, (nc + 31) / 32), block(32, 8);
    if (grid.y > 65535) return cudaErrorInvalidValue;
    if (is_float)
        plane_transpose_kernel<float><<<grid, block, 0, s>>>((const float*)src, nc, ne, dst);
    else
        plane_transpose_kernel<double><<<grid, block, 0, s>>>((const double*)src, nc, ne, dst);
    return cudaGetLastError();
}

// x[i] as float pairs (hi, lo), hi + lo = x[i] to ~48 bits: hi = x rounded to float, lo =
// the exact remainder x - hi rounded to float (the host's split, done on the device, so that
// an energy list goes up once, as doubles).
__global__ void __launch_bounds__(256)
    split_pairs_kernel(const double* __restrict__ x, int n, float2* __restrict__ out) {
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = __double2float_rn(v);
    out[i] = make_float2(h, __double2float_rn(v - (double)h));
}

cudaError_t launch_split_pairs(const double* x, int n, float2* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    split_pairs_kernel<<<(n + 255) / 256, 256, 0, s>>>(x, n, out);
    return cudaGetLastError();
}

cudaError_t launch_beam_mixed(const OscParams& p, const float2* energies, int ne, double rho_e,
                              double L_km, float* out, cudaStream_t s) {
    if (ne <= 0) return cudaSuccess;
    const float Lh = (float)L_km, rh = (float)rho_e;
    const float2 L = make_float2(Lh, (float)(L_km - (double)Lh));
    const float2 rho2 = make_float2(rh, (float)(rho_e - (double)rh));
    beam_mixed_kernel<<<(ne + kBlock - 1) / kBlock, kBlock, 0, s>>>(p, wparams(p), energies, ne,
                                                                    rho2, L, out);
    return cudaGetLastError();
}

}  // namespace cp3

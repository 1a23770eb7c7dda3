// cp3_atmos.cu -- per-bin kernels: atmospheric FP64 and mixed, beam mixed.
//
// Mapping: one CTA = one cosine row x a tile of kBlock consecutive energies, one thread =
// one (cosine, energy) bin.  The row's trajectory (segment lengths and density classes,
// a few hundred bytes) is staged in shared memory; every thread of the CTA then walks the
// same segment list, so control flow is uniform.  The per-(class, energy) eigen tables are
// read with unit stride across a warp (SoA layout) and stay L2-resident.  The result
// [9][n_cosines][n_energies] is written one channel plane at a time: each warp store is
// 32 consecutive elements (128 B in FP32, 256 B in FP64).
#include "cp3_device.cuh"
#include "cp3_kernels.hpp"
#include "cp3_mixed.cuh"

namespace cp3 {

namespace {

constexpr int kBlock = 128;
constexpr int kMaxGridY = 65535;

// ------------------------------------------------------------------------------------
// FP64: physics::calculate_atmos (physics.hpp:789-1150) for the fixed production height.

struct cm3 {
    cd a[3][3];
};

__device__ __forceinline__ void mul3(const cm3& A, const cm3& B, cm3& R) {
    // math::multiply_complex_matrix (math.hpp:84-96): R = A . B, summed over k in order.
    cm3 t;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double re = 0.0, im = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                re += A.a[i][k].re * B.a[k][j].re - A.a[i][k].im * B.a[k][j].im;
                im += A.a[i][k].im * B.a[k][j].re + A.a[i][k].re * B.a[k][j].im;
            }
            t.a[i][j] = cd{re, im};
        }
    R = t;
}

// T = sum_k e^{i arg_k} C_k for one segment (multiply_phase_matrix, math.hpp:59-75), with
// arg_k = -2.534 dmMatVac[k][0] L / E evaluated as in getArg (physics.hpp:439-450).
__device__ __forceinline__ void segment_matrix_f64(const double* __restrict__ t, int ne_pad,
                                                   double L, double E, cm3& T) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) T.a[i][j] = cd{0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double dmv = __ldg(t + (size_t)(54 + k) * ne_pad);
        double s, c;
        sincos(-kLoEFac * dmv * L / E, &s, &c);
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const double re = __ldg(t + (size_t)((k * 9 + q) * 2) * ne_pad);
            const double im = __ldg(t + (size_t)((k * 9 + q) * 2 + 1) * ne_pad);
            T.a[q / 3][q % 3].re += c * re - s * im;
            T.a[q / 3][q % 3].im += c * im + s * re;
        }
    }
}

// Production-height averaging (physics.hpp:997-1067), the reference's shift factors for the
// pairs (k, q) = (1,0), (2,0), (2,1) and each initial flavour f: sf[pair][f] = sum over bins
// of prob * sinc(d hw / 2) e^{i d hm}, d = darg0[k] - darg0[q]; the diagonal is 1.
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

// Probabilities from fin and the air layer's projectors (physics.hpp:1102-1130); with
// averaging the cross terms carry the shift factors, without they carry 1 + 0i.
template <class CatmFn>
__device__ __forceinline__ void store_prob_f64(const cm3& fin, CatmFn catm, const cd (*sf)[3],
                                               double* __restrict__ out, size_t plane) {
    const int pair[3][3] = {{-1, -1, -1}, {0, -1, -1}, {1, 2, -1}};  // (k, q) -> index, q < k
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            cd P[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double re = 0.0, im = 0.0;
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    const cd c = catm(k, q, j);
                    re += fin.a[i][q].re * c.re - fin.a[i][q].im * c.im;
                    im += fin.a[i][q].im * c.re + fin.a[i][q].re * c.im;
                }
                P[k] = cd{re, im};
            }
            double prob = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                prob += P[k].re * P[k].re + P[k].im * P[k].im;
#pragma unroll
                for (int q = 0; q < k; q++) {
                    if (sf) {
                        const cd t = sf[pair[k][q]][j];
                        prob += 2. * P[q].re * P[k].re * t.re + 2. * P[q].im * P[k].im * t.re +
                                2. * P[q].im * P[k].re * t.im - 2. * P[q].re * P[k].im * t.im;
                    } else {
                        prob += 2. * P[q].re * P[k].re + 2. * P[q].im * P[k].im;  // shift 1 + 0i
                    }
                }
            }
            // Prob[i][j] (i final, j initial) is P(j -> i): channel j*3+i.
            out[(size_t)(j * 3 + i) * plane] = prob;
        }
}

// T = sum_k e^{i arg_k} C_k for a segment of its own density (quadratic model): the
// reference's per-segment getMfast + get_product + getC, then the same phase sum.
__device__ __forceinline__ void segment_matrix_inline_f64(const OscParams* __restrict__ p, double E,
                                                          double rho, double L, cm3& T) {
    double mm[3];
    matter_masses_f64(p, E, rho, mm);
    cd C[3][3][3];
    flavour_projectors_f64(p, E, rho, mm, C);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) T.a[i][j] = cd{0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double s, c;
        sincos(-kLoEFac * (mm[k] - p->dm[0]) * L / E, &s, &c);
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const cd v = C[k][q / 3][q % 3];
            T.a[q / 3][q % 3].re += c * v.re - s * v.im;
            T.a[q / 3][q % 3].im += c * v.im + s * v.re;
        }
    }
}

// FP64 atmospheric bins, quadratic density: every segment carries its own density.
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
    const double E = energies[ie];
    const int M = nseg - 1;
    cm3 fin, mantle, T;
    segment_matrix_inline_f64(&p, E, s_rho[0], s_len[0], fin);
    for (int l = 1; l <= M; l++) {
        segment_matrix_inline_f64(&p, E, s_rho[l], s_len[l], T);
        mul3(T, fin, fin);
        if (l < M) {
            if (l == 1)
                mantle = T;
            else
                mul3(mantle, T, mantle);
        }
    }
    if (M >= 2) mul3(mantle, fin, fin);
    double mm[3];
    matter_masses_f64(&p, E, s_rho[0], mm);
    cd Catm[3][3][3];
    flavour_projectors_f64(&p, E, s_rho[0], mm, Catm);
    auto catm = [&](int k, int q, int j) { return Catm[k][q][j]; };
    double* o = out + (size_t)ic * ne + ie;
    if (av.nb > 0) {
        double arg0[3];
#pragma unroll
        for (int k = 0; k < 3; k++) arg0[k] = -kLoEFac * (mm[k] - p.dm[0]) * s_len[0] / E;
        cd sf[3][3];
        avg_shift_factors(av, ic, nc, ie, ne, arg0, sf);
        store_prob_f64(fin, catm, sf, o, (size_t)nc * ne);
    } else {
        store_prob_f64(fin, catm, (const cd(*)[3]) nullptr, o, (size_t)nc * ne);
    }
}

__global__ void __launch_bounds__(kBlock)
    atmos_f64_kernel(const double* __restrict__ energies, int ne, int ne_pad,
                     const double* __restrict__ table, const int* __restrict__ seg_off,
                     const double* __restrict__ seg_len, const int* __restrict__ seg_cls,
                     int ic0, int nc, AvgInput av, double* __restrict__ out) {
    __shared__ double s_len[kMaxSegments];
    __shared__ int s_cls[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) {
        s_len[i] = seg_len[s0 + i];
        s_cls[i] = seg_cls[s0 + i];
    }
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie];
    const size_t cls_stride = (size_t)kF64Fields * ne_pad;
    const double* tab = table + ie;
    const int M = nseg - 1;

    cm3 fin, mantle, T;
    segment_matrix_f64(tab + s_cls[0] * cls_stride, ne_pad, s_len[0], E, fin);
    for (int l = 1; l <= M; l++) {
        segment_matrix_f64(tab + s_cls[l] * cls_stride, ne_pad, s_len[l], E, T);
        mul3(T, fin, fin);
        if (l < M) {
            if (l == 1)
                mantle = T;  // identity . T is exact
            else
                mul3(mantle, T, mantle);
        }
    }
    if (M >= 2) mul3(mantle, fin, fin);

    // Probabilities: Product_k = fin . C_atm[k] with the air layer's projectors from the table.
    const double* ta = tab + s_cls[0] * cls_stride;
    auto catm = [&](int k, int q, int j) {
        return cd{__ldg(ta + (size_t)((k * 9 + q * 3 + j) * 2) * ne_pad),
                  __ldg(ta + (size_t)((k * 9 + q * 3 + j) * 2 + 1) * ne_pad)};
    };
    double* o = out + (size_t)ic * ne + ie;
    if (av.nb > 0) {
        double arg0[3];
#pragma unroll
        for (int k = 0; k < 3; k++) arg0[k] = -kLoEFac * __ldg(ta + (size_t)(54 + k) * ne_pad) * s_len[0] / E;
        cd sf[3][3];
        avg_shift_factors(av, ic, nc, ie, ne, arg0, sf);
        store_prob_f64(fin, catm, sf, o, (size_t)nc * ne);
    } else {
        store_prob_f64(fin, catm, (const cd(*)[3]) nullptr, o, (size_t)nc * ne);
    }
}

// Mixed atmospheric bins (the physics of calculate_atmos rearranged for FP32: see
// cp3_mixed.cuh).
__global__ void __launch_bounds__(kBlock)
    atmos_mixed_kernel(WParams w, const float* __restrict__ table, int ne, int ne_pad,
                       const int* __restrict__ seg_off, const float2* __restrict__ seg_len,
                       const int* __restrict__ seg_cls, int ic0, int nc, float* __restrict__ out) {
    __shared__ float2 s_len[kMaxSegments];
    __shared__ int s_cls[kMaxSegments];
    const int ic = ic0 + blockIdx.y;
    const int s0 = seg_off[ic];
    const int nseg = seg_off[ic + 1] - s0;
    for (int i = threadIdx.x; i < nseg; i += kBlock) {
        s_len[i] = seg_len[s0 + i];
        s_cls[i] = seg_cls[s0 + i];
    }
    __syncthreads();
    const int ie = blockIdx.x * kBlock + threadIdx.x;
    if (ie >= ne) return;
    atmos_bin_mixed(table + (size_t)ie * kMixFields, (size_t)kMixFields * ne_pad, s_len, s_cls,
                    nseg - 1, w, out + (size_t)ic * ne + ie, (size_t)nc * ne);
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
                             const int* seg_cls, int n_cosines, const AvgArrays& avg, double* out,
                             cudaStream_t s, RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const int ne_pad = pad_energies(ne);
    const AvgInput av{avg.prob, avg.shift, avg.air_cm, avg.n_bins, p.anti};
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        atmos_f64_kernel<<<grid, kBlock, 0, s>>>(energies, ne, ne_pad, table, seg_off, seg_len,
                                                 seg_cls, ic0, n_cosines, av, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_atmos_mixed(const OscParams& p, const float* table, int ne,
                               const int* seg_off, const float2* seg_len, const int* seg_cls,
                               int n_cosines, float* out, cudaStream_t s, RowRange rr) {
    if (ne <= 0 || n_cosines <= 0) return cudaSuccess;
    const int ne_pad = pad_energies(ne);
    const WParams w = wparams(p);
    const int end = rr.end < 0 ? n_cosines : rr.end;
    for (int ic0 = rr.begin; ic0 < end; ic0 += kMaxGridY) {
        const int rows = end - ic0 < kMaxGridY ? end - ic0 : kMaxGridY;
        dim3 grid((ne + kBlock - 1) / kBlock, rows);
        atmos_mixed_kernel<<<grid, kBlock, 0, s>>>(w, table, ne, ne_pad, seg_off, seg_len,
                                                   seg_cls, ic0, n_cosines, out);
    }
    return cudaGetLastError();
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

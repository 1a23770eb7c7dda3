// cp3_kernels.hpp -- launch wrappers of the kernels (host-callable, no CUDA types beyond
// cudaStream_t), shared by the C ABI and the batched driver.
#pragma once

#include <cuda_runtime.h>

#include "cp3_types.h"

namespace cp3 {

// Fields of one (density class, energy) entry of the eigen tables.
constexpr int kF64Fields = 10;  // u1 (3), u2 (3) rotated-basis unit eigenvectors,
                                // dmMatVac[k][0] (3), 1 unused (one 80-byte entry)
constexpr int kMixFields = 12;  // u1 (3), u2 (3) real unit eigenvectors; omega_1, omega_2 in
                                // turns per km, double-float as (hi1, hi2, lo1, lo2); 2 unused
                                // (one 48-byte entry per (class, energy))

inline int pad_energies(int ne) { return (ne + 31) / 32 * 32; }

// Eigen tables over (class, energy): FP64 flavour projectors (reference expansion), or the
// rotated-basis real projectors + double-float phase rates of the mixed kernels.
cudaError_t launch_table_f64(const OscParams& p, const double* energies, int ne,
                             const double* cls_rho, int ncls, double* table, cudaStream_t s);
cudaError_t launch_table_mixed(const OscParams& p, const double* energies, int ne,
                               const double* cls_rho, int ncls, float* table, cudaStream_t s);
// The same from float pairs (hi, lo) split on the host: no FP64 instruction on the device.
cudaError_t launch_table_mixed(const OscParams& p, const float2* energies, int ne,
                               const float2* cls_rho, int ncls, float* table, cudaStream_t s);

// Loads the mixed table kernel (the double-input instance) and the mixed per-bin kernel
// into the current device's context, as their first launch would.  With lazy module
// loading that first load may allocate device memory; a caller that must not allocate
// later (cp3_atmos_mixed_noalloc) calls these once, at set-up.
cudaError_t preload_table_mixed();
cudaError_t preload_atmos_mixed();

// Production-height averaging inputs of the FP64 kernels (n_bins == 0: fixed height).
struct AvgArrays {
    const double* prob = nullptr;    // [2][3][ne][nc][n_bins]
    const double* shift = nullptr;   // [nc][n_bins + 1] path-length shifts at the edges, cm
    const double* air_cm = nullptr;  // [nc] first (air) segment, cm
    int n_bins = 0;
};

// Cosine rows [begin, end) of a result (end < 0: through the last row).
struct RowRange {
    int begin = 0, end = -1;
};

// Atmospheric bins of an n_cosines-row result ([9][n_cosines][ne]), rows rr only.  The
// trajectory of row i is segments seg_off[i]..seg_off[i+1]-1 (air, then shells inwards); the
// table class of a row's segment l is l itself (class 0 the air, class l shell l-1, as
// build_trajectories numbers them), so no class array is read.
cudaError_t launch_atmos_f64(const OscParams& p, const double* energies, int ne,
                             const double* table, const int* seg_off, const double* seg_len,
                             int n_cosines, const AvgArrays& avg, double* out,
                             cudaStream_t s, RowRange rr = RowRange{});
cudaError_t launch_atmos_mixed(const OscParams& p, const float* table, int ne,
                               const int* seg_off, const float2* seg_len, int n_cosines,
                               float* out, cudaStream_t s,
                               RowRange rr = RowRange{});

// Production-height averaging inputs of the mixed kernels (float, from AvgArrays on the host).
struct AvgMixed {
    const float* prob = nullptr;  // [2][3][ne][nc][n_bins]
    const float2* hm = nullptr;   // [nc][n_bins] mid shift of each bin, km, float pair (0 where the
                                  // air segment has zero length)
    const float* hw = nullptr;    // [nc][n_bins] bin width, km (0 likewise)
    int nb = 0, type = 0;
};

// Mixed atmospheric bins with production-height averaging.
cudaError_t launch_atmos_mixed_avg(const OscParams& p, const float* table, int ne,
                                   const int* seg_off, const float2* seg_len, int n_cosines,
                                   const AvgMixed& av, float* out, cudaStream_t s,
                                   RowRange rr = RowRange{});

// Mixed averaged bins with the quadratic density model (per-segment eigen-solve).
cudaError_t launch_atmos_mixed_inline_avg(const OscParams& p, const double* energies, int ne,
                                          const int* seg_off, const float2* seg_len,
                                          const double* seg_rho, int n_cosines,
                                          const AvgMixed& av, float* out, cudaStream_t s,
                                          RowRange rr = RowRange{});

// Atmospheric bins whose segments each carry their own electron density (quadratic model):
// per-segment eigen-solve.  seg_len: double[] (FP64) or float2[] hi/lo (mixed).
cudaError_t launch_atmos_inline(const OscParams& p, bool mixed, const double* energies, int ne,
                                const int* seg_off, const void* seg_len, const double* seg_rho,
                                int n_cosines, const AvgArrays& avg, void* out, cudaStream_t s,
                                RowRange rr = RowRange{});

// out[i] = (x[i] rounded to float, the remainder rounded to float), on the device.
cudaError_t launch_split_pairs(const double* x, int n, float2* out, cudaStream_t s);

// One channel plane [nc][ne] (float or double) transposed to [ne][nc] doubles.
cudaError_t launch_plane_transpose(const void* src, bool is_float, int nc, int ne, double* dst,
                                   cudaStream_t s);

// Beam bins: rho_e = rho * 0.5 (electron density), L in km.
cudaError_t launch_beam_f64(const OscParams& p, const double* energies, int ne, double rho_e,
                            double L_km, double* out, cudaStream_t s);
cudaError_t launch_beam_mixed(const OscParams& p, const float2* energies, int ne, double rho_e,
                              double L_km, float* out, cudaStream_t s);

}  // namespace cp3

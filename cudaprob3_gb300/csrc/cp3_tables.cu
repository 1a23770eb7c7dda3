// cp3_tables.cu -- FP64 eigen work: the per-(density class, energy) tables of the
// atmospheric kernels and the per-bin FP64 beam kernel.
//
// This translation unit is compiled with -fmad=false: its arithmetic is the reference's
// (physics.hpp getMfast / get_product / getC / getA) in the reference's order, and keeping
// multiply and add separately rounded reproduces the reference's x86 results to the last
// bits where the eigen-system is ill-conditioned.  The table work is O(classes x energies),
// amortised over every cosine, so the missing contraction costs nothing that matters.
#include "cp3_device.cuh"
#include "cp3_f64.cuh"
#include "cp3_mixed.cuh"
#include "cp3_kernels.hpp"

namespace cp3 {

namespace {

constexpr int kTableBlock = 128;

// FP64 table: the rotated-basis unit eigenvectors u1, u2 (from the reference's getMfast
// masses, physics.hpp:267-340, and the projectors of H0 + V e0 e0^T) and dmMatVac[k][0]
// (physics.hpp:337-339), from which the bin kernel forms the reference's phases.  AoS: one
// 80-byte entry per (class c, energy e) at table[(c * ne_pad + e) * 10].
__global__ void __launch_bounds__(kTableBlock)
    table_f64_kernel(const __grid_constant__ OscParams p, const double* __restrict__ energies,
                     int ne, int ne_pad, const double* __restrict__ cls_rho,
                     double* __restrict__ table) {
    const int ie = blockIdx.x * kTableBlock + threadIdx.x;
    const int c = blockIdx.y;
    if (ie >= ne) return;
    double u[2][3], dmv[3];
    rotated_layer_f64(&p, energies[ie], cls_rho[c], u, dmv);
    double2* t = reinterpret_cast<double2*>(table + ((size_t)c * ne_pad + ie) * kF64Fields);
    t[0] = make_double2(u[0][0], u[0][1]);
    t[1] = make_double2(u[0][2], u[1][0]);
    t[2] = make_double2(u[1][1], u[1][2]);
    t[3] = make_double2(dmv[0], dmv[1]);
    t[4] = make_double2(dmv[2], 0.0);
}

// Mixed table: real unit eigenvectors u1, u2 of H0 + V e0 e0^T (P_k = u_k u_k^T) and the
// phase rates omega_k = 2.534 (m_k - m_0) / E as float pairs (rotated_eigen_vectors: FP32
// roots refined in double-float; FP64 only where two roots nearly coincide).  One 48-byte
// entry per (class c, energy e) at table[(c * ne_pad + e) * 12]: u1, u2, omega_1 hi/lo,
// omega_2 hi/lo, 2 unused -- three 16-byte words a thread reads with vector loads.
// Real = double (split on the device) or float2 (pairs split on the host: no FP64 at all).
template <class Real>
__global__ void __launch_bounds__(kTableBlock)
    table_mixed_kernel(const __grid_constant__ OscParams p, const Real* __restrict__ energies,
                       int ne, int ne_pad, const Real* __restrict__ cls_rho,
                       float* __restrict__ table) {
    const int ie = blockIdx.x * kTableBlock + threadIdx.x;
    const int c = blockIdx.y;
    if (ie >= ne) return;
    float u[2][3], om[2][2];
    rotated_eigen_vectors(&p, to_df(energies[ie]), to_df(cls_rho[c]), u, om);
    store_table_entry(table + ((size_t)c * ne_pad + ie) * kMixFields, u, om);
}

// physics::calculate_beam (physics.hpp:1153-1260), one thread per energy; result [9][ne].
// The FP64 atmospheric kernels' algebra with one segment: the reference's matter masses
// (getMfast, in this unit's uncontracted arithmetic), the rotated-basis unit eigenvectors,
// the reference's phases -2.534 dmMatVac[k][0] L / E (getA, physics.hpp:547-551) as relative
// phases, S = 1 + z1 u1 u1^T + z2 u2 u2^T and A = W S W^+.  The reference instead sums
// e^{i arg_k} times its spectral products (get_product: 18 divisions) and rotates them with
// AXFAC (getA); the two agree to rounding.
__global__ void __launch_bounds__(kTableBlock)
    beam_f64_kernel(const __grid_constant__ OscParams p, const double* __restrict__ energies,
                    int ne, double rho_e, double L, double* __restrict__ out) {
    const int ie = blockIdx.x * kTableBlock + threadIdx.x;
    if (ie >= ne) return;
    const double E = energies[ie];
    Layer64 f;
    double dmv[3], arg[3];
    rotated_layer_f64(&p, E, rho_e, f.u, dmv);
    layer64_phases(dmv, L, E, 1.0 / E, f, arg);
    layer_store64(layer_coefficients64(f.u, p.w), f.z, out + ie, (size_t)ne);
}

}  // namespace

cudaError_t launch_table_f64(const OscParams& p, const double* energies, int ne,
                             const double* cls_rho, int ncls, double* table, cudaStream_t s) {
    if (ne <= 0 || ncls <= 0) return cudaSuccess;
    dim3 grid((ne + kTableBlock - 1) / kTableBlock, ncls);
    table_f64_kernel<<<grid, kTableBlock, 0, s>>>(p, energies, ne, pad_energies(ne), cls_rho, table);
    return cudaGetLastError();
}

template <class Real>
static cudaError_t table_mixed(const OscParams& p, const Real* energies, int ne,
                               const Real* cls_rho, int ncls, float* table, cudaStream_t s) {
    if (ne <= 0 || ncls <= 0) return cudaSuccess;
    dim3 grid((ne + kTableBlock - 1) / kTableBlock, ncls);
    table_mixed_kernel<Real><<<grid, kTableBlock, 0, s>>>(p, energies, ne, pad_energies(ne), cls_rho, table);
    return cudaGetLastError();
}

cudaError_t launch_table_mixed(const OscParams& p, const double* energies, int ne,
                               const double* cls_rho, int ncls, float* table, cudaStream_t s) {
    return table_mixed(p, energies, ne, cls_rho, ncls, table, s);
}

cudaError_t launch_table_mixed(const OscParams& p, const float2* energies, int ne,
                               const float2* cls_rho, int ncls, float* table, cudaStream_t s) {
    return table_mixed(p, energies, ne, cls_rho, ncls, table, s);
}

cudaError_t preload_table_mixed() {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, table_mixed_kernel<double>);
}

cudaError_t launch_beam_f64(const OscParams& p, const double* energies, int ne, double rho_e,
                            double L_km, double* out, cudaStream_t s) {
    if (ne <= 0) return cudaSuccess;
    beam_f64_kernel<<<(ne + kTableBlock - 1) / kTableBlock, kTableBlock, 0, s>>>(p, energies, ne,
                                                                                rho_e, L_km, out);
    return cudaGetLastError();
}

}  // namespace cp3

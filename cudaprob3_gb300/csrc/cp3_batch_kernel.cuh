// cp3_batch_kernel.cuh -- the persistent many-problem kernel, shared by batches
// (cp3_batch.cu) and the serving loop (cp3_serve.cu).  See cp3_batch.cu for the design.
#pragma once

#include "cp3_mixed.cuh"

namespace cp3 {
namespace batchk {

constexpr int kTileE = 128;             // energies per atmospheric tile row
constexpr long long kSpinLimit = 20000000;  // ~seconds with the nanosleep back-off

struct Problem {
    int kind;          // 0 atmospheric, 1 beam
    int ne, ne_pad;
    int nrows;         // atmospheric: cosines; beam: baselines
    int ncls;          // atmospheric: density classes
    int param;         // index into the parameter arena
    long long e_off;   // energies arena (doubles)
    long long row_off; // atmospheric: first of nrows + 1 row offsets; beam: first baseline
    long long cls_off; // atmospheric: first class density
    long long tab_off; // atmospheric: float offset of the table [ncls][ne_pad][16]
    long long out_off; // float offset of the result
    double rho_e;      // beam: electron density (rho * 0.5)
};

struct Header {
    int nprob;
    int beam_chunk;
    long long total_a, total_b;
};

struct Args {
    const Header* hdr;
    const Problem* probs;
    const long long* a_start;  // nprob + 1 (table tiles)
    const long long* b_start;  // nprob + 1 (bin tiles)
    const OscParams* params;
    const double* energies;
    const int* row_off;
    const float2* seg_len;
    const int* seg_cls;
    const double* cls_rho;
    const float2* baselines;
    float* tables;
    float* out;
    int* done_a;
    unsigned long long* counter;
    int* status;
};

// Largest p with prefix[p] <= t (prefix[n] = total > t); skips empty ranges.
__device__ __forceinline__ int find_problem(const long long* __restrict__ prefix, int n, long long t) {
    int lo = 0, hi = n;  // invariant: prefix[lo] <= t < prefix[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

template <int R>
// 64 registers per thread (the budget of the standalone per-bin kernel): 8 blocks of 128
// or 4 of 256 threads per SM.
__global__ void __launch_bounds__(128 * R, 8 / R) batch_kernel(const Args a) {
    constexpr int T = 128 * R;
    __shared__ long long s_tile;
    __shared__ float2 s_len[R][kMaxSegments];
    __shared__ int s_cls[R][kMaxSegments];
    const int r = threadIdx.x >> 7;
    const int lane = threadIdx.x & 127;
    const Header hdr = *a.hdr;
    const long long total = hdr.total_a + hdr.total_b;
    for (;;) {
        __syncthreads();  // previous tile finished with the shared staging
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(a.counter, 1ULL);
        __syncthreads();
        const long long t = s_tile;
        if (t >= total) return;
        if (t < hdr.total_a) {
            // ---- eigen-table tile: R classes x 128 energies of one atmospheric problem ----
            const int p = find_problem(a.a_start, hdr.nprob, t);
            const Problem P = a.probs[p];
            const long long local = t - a.a_start[p];
            const int nchunk = (P.ne + kTileE - 1) / kTileE;
            const int c = (int)(local / nchunk) * R + r;
            const int e = (int)(local % nchunk) * kTileE + lane;
            if (c < P.ncls && e < P.ne) {
                float Pp[2][6], om[2][2];
                rotated_eigen_mixed(a.params + P.param, a.energies[P.e_off + e],
                                    a.cls_rho[P.cls_off + c], Pp, om);
                float4* d = reinterpret_cast<float4*>(a.tables + P.tab_off +
                                                      ((size_t)c * P.ne_pad + e) * kMixFields);
                d[0] = make_float4(Pp[0][0], Pp[0][1], Pp[0][2], Pp[0][3]);
                d[1] = make_float4(Pp[0][4], Pp[0][5], Pp[1][0], Pp[1][1]);
                d[2] = make_float4(Pp[1][2], Pp[1][3], Pp[1][4], Pp[1][5]);
                d[3] = make_float4(om[0][0], om[0][1], om[1][0], om[1][1]);
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(a.done_a + p, 1);
            continue;
        }
        // ---- bin tile --------------------------------------------------------------------
        const long long tb = t - hdr.total_a;
        const int p = find_problem(a.b_start, hdr.nprob, tb);
        const Problem P = a.probs[p];
        const long long local = tb - a.b_start[p];
        const OscParams* prm = a.params + P.param;
        const WParams w{(float)prm->w[0], (float)prm->w[1], (float)prm->w[2], (float)prm->w[3]};
        if (P.kind == 0) {
            if (threadIdx.x == 0) {
                const int need = (int)(a.a_start[p + 1] - a.a_start[p]);
                const volatile int* done = a.done_a + p;
                long long it = 0;
                while (*done < need) {
                    __nanosleep(256);
                    if (++it > kSpinLimit) {
                        atomicExch(a.status, 1);  // tables never completed: report, do not hang
                        break;
                    }
                }
                __threadfence();
            }
            const int nchunk = (P.ne + kTileE - 1) / kTileE;
            const int ic = (int)(local / nchunk) * R + r;
            const int e = (int)(local % nchunk) * kTileE + lane;
            int nseg = 0;
            if (ic < P.nrows) {
                const int s0 = a.row_off[P.row_off + ic];
                nseg = a.row_off[P.row_off + ic + 1] - s0;
                for (int i = lane; i < nseg; i += 128) {
                    s_len[r][i] = a.seg_len[s0 + i];
                    s_cls[r][i] = a.seg_cls[s0 + i];
                }
            }
            __syncthreads();
            if (ic < P.nrows && e < P.ne)
                atmos_bin_mixed<true>(a.tables + P.tab_off + (size_t)e * kMixFields,
                                      (size_t)kMixFields * P.ne_pad, s_len[r], s_cls[r], nseg - 1,
                                      w, a.out + P.out_off + (size_t)ic * P.ne + e,
                                      (size_t)P.nrows * P.ne);
        } else {
            const long long e0 = local * (long long)T * hdr.beam_chunk;
            for (int k = 0; k < hdr.beam_chunk; k++) {
                const long long e = e0 + (long long)k * T + threadIdx.x;
                if (e < P.ne)
                    beam_bin_mixed(prm, w, a.energies[P.e_off + e], P.rho_e, a.baselines + P.row_off,
                                   P.nrows, a.out + P.out_off + e, (size_t)P.ne, (size_t)9 * P.ne);
            }
        }
    }
}


}  // namespace batchk
}  // namespace cp3

// cp3_batch_kernel.cuh -- the persistent many-problem kernel, shared by batches
// (cp3_batch.cu) and the serving loop (cp3_serve.cu).  See cp3_batch.cu for the design.
//
// Scheduling is per warp, not per block: every warp pulls its own tiles from a shared
// counter (the next tile's index is fetched while the current one runs) and never waits at a
// block barrier.  A tile is 32 energies, one per lane:
//   * table tile:        one density class of one atmospheric problem;
//   * atmospheric tile:  rows_per_tile cosine rows, walked one after the other;
//   * beam tile:         beam_chunk consecutive groups of 32 energies, every baseline.
// Each warp stages the trajectory it is walking (its segment lengths) in its own
// slice of shared memory; warps synchronise only with themselves (__syncwarp).
#pragma once

#include "cp3_mixed.cuh"

namespace cp3 {
namespace batchk {

constexpr int kTileE = 32;                  // energies per tile (one per lane)
constexpr int kBlock = 128;                 // threads per block (4 independent warps)
constexpr int kMaxRowsPerTile = 16;
constexpr int kMaxBeamChunk = 64;
// A bin tile's wait for its problem's eigen tables is bounded by time (the global timer) and,
// as a backstop, by a poll count: after kWaitLimitNs the warp reports kStatusWaitLimit and
// goes on, so a launch always ends and the context stays usable.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s
constexpr long long kSpinLimit = 20000000;
// Tile indices are 32-bit: a launch holds fewer tiles than this (every warp also takes one
// index past the end).  At 32 bins per tile that is far more output than device memory.
constexpr long long kMaxTiles = (1LL << 31) - (1LL << 24);

struct Problem {
    int kind;          // 0 atmospheric, 1 beam
    int ne, ne_pad;
    int nrows;         // atmospheric: cosines; beam: baselines
    int ncls;          // atmospheric: density classes
    int param;         // index into the parameter arena
    long long e_off;   // energies arena
    long long row_off; // atmospheric: first of nrows + 1 row offsets; beam: first baseline
    long long cls_off; // atmospheric: first class density
    long long tab_off; // atmospheric: float offset of the table [ncls][ne_pad][12]
    long long out_off; // float offset of the result
    float rho_e[2];    // beam: electron density (rho * 0.5) as a float pair (hi, lo)
};

struct Header {
    int nprob;
    int rows_per_tile;
    int beam_chunk;
    int total_a, total_b;  // table tiles, bin tiles
};

struct Args {
    const Header* hdr;
    const Problem* probs;
    const int* a_start;        // nprob + 1 (table tiles)
    const int* b_start;        // nprob + 1 (bin tiles)
    const OscParams* params;
    const float2* energies;    // float pairs (hi, lo) of the energies
    const int* row_off;
    const float2* seg_len;     // segment l of a row is density class l (0 = air)
    const float2* cls_rho;     // float pairs of the class densities rho * Ye
    const float2* baselines;
    float* tables;
    float* out;
    int* done_a;
    unsigned int* counter;
    int* status;
    // Element counts of the arenas, read only by the bounds checks of CP3_DEVICE_CHECKS builds.
    long long n_tables, n_out, n_seg, n_energies;
    // The bin tiles a kPhaseBins launch runs, counted from the first bin tile:
    // [bin_lo, min(bin_hi, total_b)).  The default is all of them; a run in pieces
    // (cp3_batch_run_to_host) launches one window of whole problems per piece.
    int bin_lo = 0, bin_hi = 0x7fffffff;
};

// Status words the kernel can leave: a wait that ran out, a tile of a kind the instance was
// not built for, and (CP3_DEVICE_CHECKS builds) a tile whose accesses would have left an
// arena, which is then skipped.
constexpr int kStatusWaitLimit = 1, kStatusKind = 2, kStatusBounds = 3;

__device__ __forceinline__ unsigned long long global_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

#ifdef CP3_DEVICE_CHECKS
// [off, off + len) inside an arena of n elements.
__device__ __forceinline__ bool span_ok(long long off, long long len, long long n) {
    return off >= 0 && len >= 0 && off + len <= n;
}
#endif

// Table and bin tiles of one problem for a tile shape.
CP3_HD void problem_tiles(const Problem& P, int rows_per_tile, int beam_chunk, long long* na,
                          long long* nb) {
    const long long nchunk = (P.ne + kTileE - 1) / kTileE;
    if (P.kind == 0) {
        *na = nchunk * P.ncls;
        *nb = nchunk * ((P.nrows + rows_per_tile - 1) / rows_per_tile);
    } else {
        const long long per = (long long)kTileE * beam_chunk;
        *na = 0;
        *nb = (P.ne + per - 1) / per;
    }
}

// Largest p in [lo, n) with prefix[p] <= t, given prefix[lo] <= t < prefix[n]; skips empty
// ranges.
__device__ __forceinline__ int find_problem(const int* __restrict__ prefix, int lo, int n, int t) {
    int hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Which problem kinds a launch contains (bit set): the kernel is compiled once per set, so a
// launch of one kind carries neither the code nor the register pressure of the other.
constexpr int kAtmos = 1, kBeam = 2, kBoth = 3;

CP3_HD int launch_kinds(bool has_atmos, bool has_beam) {
    return (has_atmos ? kAtmos : 0) | (has_beam ? kBeam : 0);
}

// Which tiles a launch runs.  kPhaseAll: table and bin tiles in one launch, each atmospheric
// bin tile waiting (bounded) for its problem's tables, which it then reads from L2 (__ldcg:
// they were written during this launch).  Split: a kPhaseTables launch, then a kPhaseBins
// launch in stream order, which needs no wait and reads tables an earlier launch wrote
// through the read-only path (__ldg).  Counter 0 serves kPhaseAll and kPhaseTables launches,
// counter 1 kPhaseBins launches.
constexpr int kPhaseTables = 1, kPhaseBins = 2, kPhaseAll = 3;

// 72 registers per thread, 7 blocks per SM: measured 1-2 % faster on the batched atmospheric
// and beam workloads than 64 registers (8 blocks), which spill more; 6 blocks is slower.  The
// kPhaseBins instance fits 72 registers without spills; 64 or 56 (8 or 9 blocks) measured
// no faster on the batched atmospheric workload.
// Internal linkage: each translation unit that launches it (batches, the server) has its own.
template <int kKinds, int kPhases = kPhaseAll>
static __global__ void __launch_bounds__(kBlock, 7) batch_kernel(const Args a) {
    constexpr int kWarps = kBlock / 32;
    constexpr int kTableLoad = kPhases == kPhaseBins ? kLoadReadOnly : kLoadL2;
    __shared__ float2 s_len[kWarps][kMaxSegments];  // one trajectory per warp
    const unsigned lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const Header hdr = *a.hdr;
    const int first = kPhases == kPhaseBins ? hdr.total_a + a.bin_lo : 0;
    const int total = kPhases == kPhaseTables ? hdr.total_a
                      : kPhases == kPhaseBins ? hdr.total_a + min(hdr.total_b, a.bin_hi)
                                              : hdr.total_a + hdr.total_b;
    unsigned int* const counter = a.counter + (kPhases == kPhaseBins ? 1 : 0);

    // The warp's current problem: tiles arrive in increasing order, so a warp's problems do
    // too and the lookup resumes from the last one.  The descriptor itself is re-read per
    // tile (a broadcast load that hits L1), which keeps registers free for the bins.
    int p = 0, phase = -1, ready = -1, p_lo = 0, p_hi = 0;

    int t = 0;
    if (lane == 0) t = first + (int)atomicAdd(counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    while (t < total) {
        int next = 0;
        if (lane == 0) next = first + (int)atomicAdd(counter, 1u);  // in flight while this tile runs

        const int ph = kPhases == kPhaseTables ? 0 : kPhases == kPhaseBins ? 1 : t < hdr.total_a ? 0 : 1;
        const int tt = ph == 0 ? t : t - hdr.total_a;
        if (ph != phase || tt >= p_hi) {
            const int* pre = ph == 0 ? a.a_start : a.b_start;
            p = find_problem(pre, ph == phase ? p : 0, hdr.nprob, tt);
            p_lo = __ldg(pre + p);
            p_hi = __ldg(pre + p + 1);
            phase = ph;
        }
        const Problem P = a.probs[p];
        const int local = tt - p_lo;
        const OscParams* prm = a.params + P.param;

        if (ph == 0) {
            if (!(kKinds & kAtmos)) {  // cannot happen: the host picks kKinds from the problems
                if (lane == 0) atomicExch(a.status, kStatusKind);
                break;
            }
            // ---- eigen-table tile: one class x 32 energies ----------------------------
            const int nchunk = (P.ne + kTileE - 1) / kTileE;
            const int c = local / nchunk;
            const int e = (local % nchunk) * kTileE + (int)lane;
#ifdef CP3_DEVICE_CHECKS
            if (!(c >= 0 && c < P.ncls && span_ok(P.e_off, P.ne, a.n_energies) &&
                  span_ok(P.tab_off, (long long)P.ncls * P.ne_pad * kMixFields, a.n_tables) &&
                  P.ne <= P.ne_pad)) {
                if (lane == 0) atomicExch(a.status, kStatusBounds);
                __syncwarp();
                if (lane == 0) atomicAdd(a.done_a + p, 1);  // no waiter is left hanging
                t = __shfl_sync(0xffffffffu, next, 0);
                continue;
            }
#endif
            if (e < P.ne) {
                float u[2][3], om[2][2];
                const float2 E2 = a.energies[P.e_off + e], r2 = a.cls_rho[P.cls_off + c];
                rotated_eigen_vectors(prm, df{E2.x, E2.y}, df{r2.x, r2.y}, u, om);
                store_table_entry(a.tables + P.tab_off + ((size_t)c * P.ne_pad + e) * kMixFields,
                                  u, om);
            }
            __threadfence();
            __syncwarp();
            if (lane == 0) atomicAdd(a.done_a + p, 1);
        } else if (P.kind == 0) {
            if (!(kKinds & kAtmos)) {
                if (lane == 0) atomicExch(a.status, kStatusKind);
                break;
            }
            // ---- atmospheric bin tile: rows_per_tile rows x 32 energies ------------------
            if (kPhases == kPhaseAll && ready != p) {
                // This problem's table tiles were all handed out before this tile, to warps
                // that are running them, so the wait ends; it is bounded all the same.
                if (lane == 0) {
                    const int need = __ldg(a.a_start + p + 1) - __ldg(a.a_start + p);
                    const volatile int* done = a.done_a + p;
                    const unsigned long long t0 = global_timer_ns();
                    long long it = 0;
                    while (*done < need) {
                        __nanosleep(256);
                        if (++it > kSpinLimit || global_timer_ns() - t0 > kWaitLimitNs) {
                            atomicExch(a.status, kStatusWaitLimit);  // tables never completed: report
                            break;
                        }
                    }
                    __threadfence();
                }
                __syncwarp();
                ready = p;
            }
            const WParams w = wparams(*prm);
            const int nchunk = (P.ne + kTileE - 1) / kTileE;
            const int ic0 = (local / nchunk) * hdr.rows_per_tile;
            const int ic1 = min(ic0 + hdr.rows_per_tile, P.nrows);
            const int e = (local % nchunk) * kTileE + (int)lane;
            const int* ro = a.row_off + P.row_off;
#ifdef CP3_DEVICE_CHECKS
            bool tile_ok = ic0 >= 0 && ic0 < P.nrows &&
                           span_ok(P.out_off, 9LL * P.nrows * P.ne, a.n_out) &&
                           span_ok(P.tab_off, (long long)P.ncls * P.ne_pad * kMixFields, a.n_tables);
#endif
            for (int ic = ic0; ic < ic1; ic++) {
                const int s0 = __ldg(ro + ic);
                const int nseg = __ldg(ro + ic + 1) - s0;
#ifdef CP3_DEVICE_CHECKS
                // segment l reads the table of class l: the row's M + 1 segments need M < ncls
                tile_ok = tile_ok && nseg >= 1 && nseg <= kMaxSegments && nseg <= P.ncls &&
                          span_ok(s0, nseg, a.n_seg);
                if (!tile_ok) {
                    if (lane == 0) atomicExch(a.status, kStatusBounds);
                    break;
                }
#endif
                __syncwarp();  // the previous row is done with the staging
                for (int i = (int)lane; i < nseg; i += 32) s_len[wid][i] = __ldg(a.seg_len + s0 + i);
                __syncwarp();
                if (e < P.ne)
                    atmos_bin_mixed<kTableLoad, true>(a.tables + P.tab_off + (size_t)e * kMixFields,
                                                      (size_t)kMixFields * P.ne_pad, s_len[wid],
                                                      nseg - 1, w,
                                                      a.out + P.out_off + (size_t)ic * P.ne + e,
                                                      (size_t)P.nrows * P.ne);
            }
        } else {
            if (!(kKinds & kBeam)) {
                if (lane == 0) atomicExch(a.status, kStatusKind);
                break;
            }
            // ---- beam tile: beam_chunk x 32 energies, every baseline --------------------
            const WParams w = wparams(*prm);
            const long long e0 = (long long)local * kTileE * hdr.beam_chunk;
            const df rho{P.rho_e[0], P.rho_e[1]};
#ifdef CP3_DEVICE_CHECKS
            if (!(span_ok(P.out_off, 9LL * P.nrows * P.ne, a.n_out) &&
                  span_ok(P.e_off, P.ne, a.n_energies))) {
                if (lane == 0) atomicExch(a.status, kStatusBounds);
                t = __shfl_sync(0xffffffffu, next, 0);
                continue;
            }
#endif
            for (int k = 0; k < hdr.beam_chunk; k++) {
                const long long e = e0 + (long long)k * kTileE + lane;
                if (e < P.ne) {
                    const float2 E2 = a.energies[P.e_off + e];
                    beam_bin_mixed(prm, w, df{E2.x, E2.y}, rho, a.baselines + P.row_off, P.nrows,
                                   a.out + P.out_off + e, (size_t)P.ne, (size_t)9 * P.ne);
                }
            }
        }
        t = __shfl_sync(0xffffffffu, next, 0);
    }
}

}  // namespace batchk
}  // namespace cp3

// cp3_mixed.cuh -- building blocks of the mixed-precision per-bin computation, shared by
// the single-problem kernels (cp3_atmos.cu) and the batched persistent kernel (cp3_batch.cu).
#pragma once

#include "cp3_device.cuh"
#include "cp3_kernels.hpp"

namespace cp3 {

// ------------------------------------------------------------------------------------
// Mixed: the same physics, rearranged for FP32.
//   T_l = W S_l W^+,  S_l = 1 + z1 u1 u1^T + z2 u2 u2^T,  z_k = e^{-i omega_k L_l} - 1,
// with u_k the real unit eigenvectors of H0 + V e0 e0^T (S_l is complex symmetric), and
//   A   = W (S_1..S_{M-1}) S_M (S_{M-1}..S_1) S_0 W^+ = W (B^T S_M B) S_0 W^+,
// with B = S_{M-1}..S_1, because S_l^T = S_l.  That is M+1 layer applications per bin
// instead of the reference's 2M-1 products; each applies S as two rank-1 updates,
// G += z_k u_k (u_k^T G), 96 FMA-pipe instructions against 132 for forming S and a
// symmetric-by-general product.

struct cs6 {  // complex symmetric 3x3
    cf a[6];
};
struct cg9 {  // complex general 3x3
    cf a[3][3];
};

// One layer in factored form.
struct Layer {
    float u[2][3];  // unit eigenvectors u1, u2
    float z[2][2];  // z_k = e^{-i omega_k L} - 1 (re, im)
};

// S = 1 + z1 P1 + z2 P2 from the two phase factors and the real projectors (beam).
__device__ __forceinline__ void layer_matrix(const float z[2][2], const float P1[6],
                                             const float P2[6], cs6& S) {
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const float one = (q == 0 || q == 3 || q == 5) ? 1.0f : 0.0f;
        S.a[q].re = fmaf(z[1][0], P2[q], fmaf(z[0][0], P1[q], one));
        S.a[q].im = fmaf(z[1][1], P2[q], z[0][1] * P1[q]);
    }
}

// How a kernel reads the eigen table: the read-only path (__ldg) for tables an earlier
// launch wrote, L2 only (__ldcg) for tables written earlier in the same launch.
enum TableLoad { kLoadReadOnly = 0, kLoadL2 = 1 };

// t points at this bin's 48-byte table entry: u1 (3), u2 (3), omega_1 (hi, lo), omega_2
// (hi, lo), 2 unused.
template <int kLoad = kLoadReadOnly>
__device__ __forceinline__ void layer_from_table(const float* __restrict__ t, float2 L, Layer& f) {
    const float4* t4 = reinterpret_cast<const float4*>(t);
    float4 a, b, c;
    if (kLoad == kLoadL2) {
        a = __ldcg(t4);
        b = __ldcg(t4 + 1);
        c = __ldcg(t4 + 2);
    } else {
        a = __ldg(t4);
        b = __ldg(t4 + 1);
        c = __ldg(t4 + 2);
    }
    f.u[0][0] = a.x;
    f.u[0][1] = a.y;
    f.u[0][2] = a.z;
    f.u[1][0] = a.w;
    f.u[1][1] = b.x;
    f.u[1][2] = b.y;
    float lo;
    float r = reduced_phase(b.z, b.w, L.x, L.y, lo);
    unit_phase_minus_one(r, lo, f.z[0][0], f.z[0][1]);
    r = reduced_phase(c.x, c.y, L.x, L.y, lo);
    unit_phase_minus_one(r, lo, f.z[1][0], f.z[1][1]);
}

// The table entry of one (class, energy): eigenvectors and phase rates, three float4.
__device__ __forceinline__ void store_table_entry(float* __restrict__ t, const float u[2][3],
                                                  const float om[2][2]) {
    float4* d = reinterpret_cast<float4*>(t);
    d[0] = make_float4(u[0][0], u[0][1], u[0][2], u[1][0]);
    d[1] = make_float4(u[1][1], u[1][2], om[0][0], om[0][1]);
    d[2] = make_float4(om[1][0], om[1][1], 0.f, 0.f);
}

// G <- S G
__device__ __forceinline__ void apply_left(const Layer& f, cg9& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float* u = f.u[k];
        const float zr = f.z[k][0], zi = f.z[k][1];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float wr = u[0] * G.a[0][j].re, wi = u[0] * G.a[0][j].im;
            wr = fmaf(u[1], G.a[1][j].re, wr);
            wi = fmaf(u[1], G.a[1][j].im, wi);
            wr = fmaf(u[2], G.a[2][j].re, wr);
            wi = fmaf(u[2], G.a[2][j].im, wi);
            const float yr = fmaf(zr, wr, -zi * wi), yi = fmaf(zr, wi, zi * wr);
#pragma unroll
            for (int i = 0; i < 3; i++) {
                G.a[i][j].re = fmaf(u[i], yr, G.a[i][j].re);
                G.a[i][j].im = fmaf(u[i], yi, G.a[i][j].im);
            }
        }
    }
}

// G <- G S
__device__ __forceinline__ void apply_right(const Layer& f, cg9& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float* u = f.u[k];
        const float zr = f.z[k][0], zi = f.z[k][1];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float wr = G.a[i][0].re * u[0], wi = G.a[i][0].im * u[0];
            wr = fmaf(G.a[i][1].re, u[1], wr);
            wi = fmaf(G.a[i][1].im, u[1], wi);
            wr = fmaf(G.a[i][2].re, u[2], wr);
            wi = fmaf(G.a[i][2].im, u[2], wi);
            const float yr = fmaf(zr, wr, -zi * wi), yi = fmaf(zr, wi, zi * wr);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                G.a[i][j].re = fmaf(yr, u[j], G.a[i][j].re);
                G.a[i][j].im = fmaf(yi, u[j], G.a[i][j].im);
            }
        }
    }
}

// G = S = 1 + z1 u1 u1^T + z2 u2 u2^T
__device__ __forceinline__ void layer_to_gen(const Layer& f, cg9& G) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const float p0 = f.u[0][i] * f.u[0][j], p1 = f.u[1][i] * f.u[1][j];
            const cf v{fmaf(f.z[1][0], p1, fmaf(f.z[0][0], p0, i == j ? 1.0f : 0.0f)),
                       fmaf(f.z[1][1], p1, f.z[0][1] * p0)};
            G.a[i][j] = v;
            G.a[j][i] = v;
        }
}

// One Newton-Schulz step toward the nearest unitary matrix, A <- A (3 - A^+ A) / 2.  The
// rounding of FP32 layer matrices leaves each slightly non-unitary and that part of the
// error accumulates over the ~2M products of a deep trajectory; one step at the end removes
// it to second order (measured: max error on the 59-shell, 2000 x 2000 grid drops by ~2x).
__device__ __forceinline__ void newton_schulz(cg9& A) {
    cg9 G;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float re = 0.f, im = 0.f;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const cf a = A.a[k][i], b = A.a[k][j];  // conj(a) b
                re = fmaf(a.re, b.re, fmaf(a.im, b.im, re));
                im = fmaf(a.re, b.im, fmaf(-a.im, b.re, im));
            }
            G.a[i][j] = cf{(i == j ? 1.5f : 0.f) - 0.5f * re, -0.5f * im};
        }
    cg9 R;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            cf acc = cmulf(A.a[i][0], G.a[0][j]);
#pragma unroll
            for (int k = 1; k < 3; k++) {
                const cf a = A.a[i][k], g = G.a[k][j];
                acc.re = fmaf(a.re, g.re, fmaf(-a.im, g.im, acc.re));
                acc.im = fmaf(a.re, g.im, fmaf(a.im, g.re, acc.im));
            }
            R.a[i][j] = acc;
        }
    A = R;
}

__device__ __forceinline__ void sym_to_gen(const cs6& S, cg9& G) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) G.a[i][j] = S.a[sidx(i, j)];
}

// Probabilities of A = W A2 W^+, W = [[1,0,0],[0,c,s e],[0,-s,c e]], e = e^{i d}; stores
// channel a*3+b = |A[b][a]|^2 at out[ch * plane].
__device__ __forceinline__ void store_probabilities(const cg9& A2, float c, float s, float ed_re,
                                                    float ed_im, float* __restrict__ out,
                                                    size_t plane) {
    cg9 Y;  // Y = A2 W^+ : columns 1, 2 mix through (c, -s) and e* (s, c)
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const cf a1 = A2.a[i][1], a2 = A2.a[i][2];
        const cf f{a2.re * ed_re + a2.im * ed_im, a2.im * ed_re - a2.re * ed_im};  // e* a2
        Y.a[i][0] = A2.a[i][0];
        Y.a[i][1] = cf{fmaf(c, a1.re, s * f.re), fmaf(c, a1.im, s * f.im)};
        Y.a[i][2] = cf{fmaf(-s, a1.re, c * f.re), fmaf(-s, a1.im, c * f.im)};
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const cf y1 = Y.a[1][j], y2 = Y.a[2][j];
        const cf g{y2.re * ed_re - y2.im * ed_im, y2.re * ed_im + y2.im * ed_re};  // e y2
        const cf r0 = Y.a[0][j];
        const cf r1{fmaf(c, y1.re, s * g.re), fmaf(c, y1.im, s * g.im)};
        const cf r2{fmaf(-s, y1.re, c * g.re), fmaf(-s, y1.im, c * g.im)};
        // column j = initial flavour j; rows 0..2 = final flavours
        out[(size_t)(j * 3 + 0) * plane] = fmaf(r0.re, r0.re, r0.im * r0.im);
        out[(size_t)(j * 3 + 1) * plane] = fmaf(r1.re, r1.re, r1.im * r1.im);
        out[(size_t)(j * 3 + 2) * plane] = fmaf(r2.re, r2.re, r2.im * r2.im);
    }
}

struct WParams {
    float c, s, er, ei;
};

CP3_HD WParams wparams(const OscParams& p) {
    return WParams{p.wf[0], p.wf[1], p.wf[2], p.wf[3]};
}

// One atmospheric bin over M+1 segments, generic in where each segment's layer comes from:
// seg(l, F) fills F for segment l (0 = air, then shells inwards).
// The bin's amplitude before the air layer, for M >= 1: G = B^T S_M B (M >= 2) or S_1 (M = 1),
// with B = S_{M-1}..S_1; seg(l, F) fills layer l.
template <class SegFn>
__device__ __forceinline__ void chain_mixed(SegFn seg, int M, cg9& G) {
    Layer F;
    seg(1, F);
    layer_to_gen(F, G);  // B = S_1
    if (M > 1) {
        cg9& B = G;
        for (int l = 2; l < M; l++) {
            seg(l, F);
            apply_left(F, B);
        }
        seg(M, F);
        cg9 X = B;
        apply_left(F, X);  // X = S_M B
        cs6 Q;             // Q = B^T X (symmetric)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) {
                cf acc = cmulf(B.a[0][i], X.a[0][j]);
#pragma unroll
                for (int k = 1; k < 3; k++) {
                    const cf b = B.a[k][i], x = X.a[k][j];
                    acc.re = fmaf(b.re, x.re, fmaf(-b.im, x.im, acc.re));
                    acc.im = fmaf(b.re, x.im, fmaf(b.im, x.re, acc.im));
                }
                Q.a[sidx(i, j)] = acc;
            }
        sym_to_gen(Q, G);
    }
}

// One atmospheric bin over M+1 segments, generic in where each segment's layer comes from:
// seg(l, F) fills F for segment l (0 = air, then shells inwards).
template <class SegFn>
__device__ __forceinline__ void atmos_bin_mixed_with(SegFn seg, int M, const WParams& w,
                                                     float* __restrict__ out, size_t plane) {
    cg9 A2;
    Layer F;
    if (M == 0) {
        seg(0, F);
        layer_to_gen(F, A2);
    } else {
        chain_mixed(seg, M, A2);
        seg(0, F);
        apply_right(F, A2);  // ... S_0
    }
    // One or two FP32 layer matrices are unitary to ~1e-7 already; the correction pays off
    // from the longer chains on (it removes the drift accumulated over ~2M products).
    if (M >= 2) newton_schulz(A2);
    store_probabilities(A2, w.c, w.s, w.er, w.ei, out, plane);
}

// One atmospheric bin from the eigen table: the trajectory's segment lengths and classes are
// in shared memory (s_len[0..M], s_cls[0..M]); tab points at this bin's energy column of the
// table (entry of class c at tab + c * cls_stride); probabilities go to out[ch * plane].
template <int kLoad = kLoadReadOnly>
__device__ __forceinline__ void atmos_bin_mixed(const float* __restrict__ tab, size_t cls_stride,
                                                const float2* s_len, const int* s_cls, int M,
                                                const WParams& w, float* __restrict__ out,
                                                size_t plane) {
    atmos_bin_mixed_with(
        [&](int l, Layer& F) { layer_from_table<kLoad>(tab + s_cls[l] * cls_stride, s_len[l], F); },
        M, w, out, plane);
}

// Layer of a segment whose density is its own (quadratic density model): the
// eigen-decomposition is solved for this segment (double-float refined).
__device__ __forceinline__ void segment_layer_inline(const OscParams* __restrict__ p, double E,
                                                     double rho_e, float2 L, Layer& f) {
    float om[2][2];
    rotated_eigen_vectors(p, df_from(E), df_from(rho_e), f.u, om);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        float lo;
        const float r = reduced_phase(om[k][0], om[k][1], L.x, L.y, lo);
        unit_phase_minus_one(r, lo, f.z[k][0], f.z[k][1]);
    }
}

// One beam energy (E, rho_e as double or float pair): eigen-decomposition (double-float
// refined), then for each baseline L[j] the layer matrix and the nine probabilities at
// out + j * baseline_stride + ch * plane.
template <class Real>
__device__ __forceinline__ void beam_bin_mixed(const OscParams* __restrict__ p, const WParams& w,
                                               Real E, Real rho_e, const float2* L, int nL,
                                               float* __restrict__ out, size_t plane,
                                               size_t baseline_stride) {
    float P[2][6], om[2][2];
    rotated_eigen_mixed(p, E, rho_e, P, om);
    for (int j = 0; j < nL; j++) {
        float z[2][2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            float lo;
            const float r = reduced_phase(om[k][0], om[k][1], L[j].x, L[j].y, lo);
            unit_phase_minus_one(r, lo, z[k][0], z[k][1]);
        }
        cs6 S;
        layer_matrix(z, P[0], P[1], S);
        cg9 A2;
        sym_to_gen(S, A2);
        store_probabilities(A2, w.c, w.s, w.er, w.ei, out + j * baseline_stride, plane);
    }
}

}  // namespace cp3

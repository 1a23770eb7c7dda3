// cp3_mixed.cuh -- building blocks of the mixed-precision per-bin computation, shared by
// the single-problem kernels (cp3_atmos.cu) and the batched persistent kernel (cp3_batch.cu).
#pragma once

#include "cp3_device.cuh"
#include "cp3_kernels.hpp"

namespace cp3 {

// ------------------------------------------------------------------------------------
// Mixed: the same physics, rearranged for FP32.
//   T_l = W S_l W^+,  S_l = 1 + z1 u1 u1^T + z2 u2 u2^T,  z_k = e^{-i omega_k L_l} - 1
// (omega_k carried in turns, omega_k / 2 pi, so that the phase reduction is exact),
// with u_k the real unit eigenvectors of H0 + V e0 e0^T (S_l is complex symmetric), and
//   A   = W (S_1..S_{M-1}) S_M (S_{M-1}..S_1) S_0 W^+ = W (B^T S_M B) S_0 W^+,
// with B = S_{M-1}..S_1, because S_l^T = S_l.  That is M+1 layer applications per bin
// instead of the reference's 2M-1 products; each applies S as two rank-1 updates,
// G += z_k u_k (u_k^T G): 96 FMAs (48 of them paired over re/im) against 132 for forming S
// and a symmetric-by-general product.

struct cg9 {  // complex general 3x3
    cf a[3][3];
};

// One layer in factored form.
struct Layer {
    float u[2][3];  // unit eigenvectors u1, u2
    float z[2][2];  // z_k = e^{-i omega_k L} - 1 (re, im)
};

// ------------------------------------------------------------------------------------
// Paired FP32 forms (bc2, neg2 and df2 are in cp3_device.cuh): complex entries as (re, im)
// lanes, and the two phases (k = 1, 2) of one layer side by side.

__device__ __forceinline__ float2 f2(cf c) { return make_float2(c.re, c.im); }
__device__ __forceinline__ cf fc(float2 v) { return cf{v.x, v.y}; }

// reduced_turn for the two phase rates (ah + al).x and (ah + al).y of one layer (turns per
// km) times the same path length bh + bl; lane for lane the same operations and roundings.
__device__ __forceinline__ float2 reduced_turn2(float2 ah, float2 al, float bh, float bl,
                                                float2& lo) {
    const float2 B = bc2(bh);
    const float2 p = __fmul2_rn(ah, B);
    float2 e = __ffma2_rn(ah, B, neg2(p));
    e = __ffma2_rn(ah, bc2(bl), e);
    e = __ffma2_rn(al, B, e);
    const float2 f = __fadd2_rn(p, make_float2(-rintf(p.x), -rintf(p.y)));  // exact
    const float2 s = __fadd2_rn(f, e);
    lo = __fadd2_rn(__fadd2_rn(f, neg2(s)), e);
    return s;
}

// poly_sincos_turns of two arguments, lane for lane.
__device__ __forceinline__ void poly_sincos_turns2(float2 x, float2& s, float2& c) {
    const float2 x2 = __fmul2_rn(x, x);
    float2 ps = __ffma2_rn(bc2(kP9), x2, bc2(kP7));
    ps = __ffma2_rn(ps, x2, bc2(kP5));
    ps = __ffma2_rn(ps, x2, bc2(kP3));
    ps = __ffma2_rn(ps, x2, bc2(kS1Lo));
    s = __ffma2_rn(x, bc2(kS1Hi), __fmul2_rn(x, ps));
    float2 pc = __ffma2_rn(bc2(kQ10), x2, bc2(kQ8));
    pc = __ffma2_rn(pc, x2, bc2(kQ6));
    pc = __ffma2_rn(pc, x2, bc2(kQ4));
    pc = __ffma2_rn(pc, x2, bc2(kC2Lo));
    c = __ffma2_rn(x2, pc, __ffma2_rn(x2, bc2(kC2Hi), bc2(1.0f)));
}

// unit_turn_minus_one of two phases, lane for lane: z_k = zre.k + i zim.k.
__device__ __forceinline__ void unit_turn_minus_one2(float2 r, float2 lo, float2& zre,
                                                     float2& zim) {
    const float2 a = make_float2(fabsf(r.x), fabsf(r.y));
    const bool rx = a.x > 0.25f, ry = a.y > 0.25f;
    const float2 t = __fadd2_rn(bc2(0.5f), neg2(a));
    float2 sx, cx;
    poly_sincos_turns2(make_float2(rx ? t.x : a.x, ry ? t.y : a.y), sx, cx);
    // sin(r) = sign(r) sin(|r|): the sign bit of r flips that of sx (one bit operation)
    const float2 sn = make_float2(
        __int_as_float(__float_as_int(sx.x) ^ (__float_as_int(r.x) & 0x80000000)),
        __int_as_float(__float_as_int(sx.y) ^ (__float_as_int(r.y) & 0x80000000)));
    const float2 cs = make_float2(rx ? -cx.x : cx.x, ry ? -cx.y : cx.y);
    const float2 ml = __fmul2_rn(lo, bc2(-kTwoPiF));
    zre = __ffma2_rn(ml, sn, __fadd2_rn(cs, bc2(-1.0f)));
    zim = __ffma2_rn(ml, cs, neg2(sn));
}

// The same with the hardware sine and cosine (sin.approx / cos.approx) of 2 pi r: absolute
// error about 4e-7 on [-pi, pi], against about an ulp for the polynomial.  For the beam's
// single layer per baseline that is an error of the same size in each probability; the
// deep atmospheric chains, where the layers' errors add up, keep the polynomial.
__device__ __forceinline__ void unit_turn_minus_one2_hw(float2 r, float2 lo, float2& zre,
                                                        float2& zim) {
    const float2 x = __fmul2_rn(r, bc2(kTwoPiF));
    float2 sn, cs;
    __sincosf(x.x, &sn.x, &cs.x);
    __sincosf(x.y, &sn.y, &cs.y);
    const float2 ml = __fmul2_rn(lo, bc2(-kTwoPiF));
    zre = __ffma2_rn(ml, sn, __fadd2_rn(cs, bc2(-1.0f)));
    zim = __ffma2_rn(ml, cs, neg2(sn));
}

// How a kernel reads the eigen table: the read-only path (__ldg) for tables an earlier
// launch wrote, L2 only (__ldcg) for tables written earlier in the same launch.
enum TableLoad { kLoadReadOnly = 0, kLoadL2 = 1 };

// t points at this bin's 48-byte table entry: u1 (3), u2 (3), then the phase rates
// omega_1, omega_2 in turns per km (omega / 2 pi) as double-floats, the two high parts side
// by side and the two low parts side by side (each pair one aligned 8-byte register pair of
// the float4 loads), 2 unused: [u1 | u2 | om1.hi om2.hi | om1.lo om2.lo | 0 0].
struct TableEntry {
    float4 a, b, c;
};

template <int kLoad = kLoadReadOnly>
__device__ __forceinline__ TableEntry load_table_entry(const float* __restrict__ t) {
    const float4* t4 = reinterpret_cast<const float4*>(t);
    if (kLoad == kLoadL2) return TableEntry{__ldcg(t4), __ldcg(t4 + 1), __ldcg(t4 + 2)};
    return TableEntry{__ldg(t4), __ldg(t4 + 1), __ldg(t4 + 2)};
}

__device__ __forceinline__ void layer_from_entry(const TableEntry& e, float2 L, Layer& f) {
    f.u[0][0] = e.a.x;
    f.u[0][1] = e.a.y;
    f.u[0][2] = e.a.z;
    f.u[1][0] = e.a.w;
    f.u[1][1] = e.b.x;
    f.u[1][2] = e.b.y;
    float2 lo, zr, zi;
    const float2 r =
        reduced_turn2(make_float2(e.b.z, e.b.w), make_float2(e.c.x, e.c.y), L.x, L.y, lo);
    unit_turn_minus_one2(r, lo, zr, zi);
    f.z[0][0] = zr.x;
    f.z[0][1] = zi.x;
    f.z[1][0] = zr.y;
    f.z[1][1] = zi.y;
}

template <int kLoad = kLoadReadOnly>
__device__ __forceinline__ void layer_from_table(const float* __restrict__ t, float2 L, Layer& f) {
    layer_from_entry(load_table_entry<kLoad>(t), L, f);
}

// The table entry of one (class, energy): eigenvectors and phase rates, three float4.
__device__ __forceinline__ void store_table_entry(float* __restrict__ t, const float u[2][3],
                                                  const float om[2][2]) {
    float4* d = reinterpret_cast<float4*>(t);
    d[0] = make_float4(u[0][0], u[0][1], u[0][2], u[1][0]);
    d[1] = make_float4(u[1][1], u[1][2], om[0][0], om[1][0]);
    d[2] = make_float4(om[0][1], om[1][1], 0.f, 0.f);
}

// G <- S G.  Per column: w = u^T G (paired over re/im), y = z w, G += u y (paired).
__device__ __forceinline__ void apply_left(const Layer& f, cg9& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float* u = f.u[k];
        const float zr = f.z[k][0], zi = f.z[k][1];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            float2 w = __fmul2_rn(bc2(u[0]), f2(G.a[0][j]));
            w = __ffma2_rn(bc2(u[1]), f2(G.a[1][j]), w);
            w = __ffma2_rn(bc2(u[2]), f2(G.a[2][j]), w);
            const float2 y = make_float2(fmaf(zr, w.x, -zi * w.y), fmaf(zr, w.y, zi * w.x));
#pragma unroll
            for (int i = 0; i < 3; i++) G.a[i][j] = fc(__ffma2_rn(bc2(u[i]), y, f2(G.a[i][j])));
        }
    }
}

// G <- G S.  Per row: w = G u, y = w z, G += y u^T.
__device__ __forceinline__ void apply_right(const Layer& f, cg9& G) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float* u = f.u[k];
        const float zr = f.z[k][0], zi = f.z[k][1];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float2 w = __fmul2_rn(f2(G.a[i][0]), bc2(u[0]));
            w = __ffma2_rn(f2(G.a[i][1]), bc2(u[1]), w);
            w = __ffma2_rn(f2(G.a[i][2]), bc2(u[2]), w);
            const float2 y = make_float2(fmaf(zr, w.x, -zi * w.y), fmaf(zr, w.y, zi * w.x));
#pragma unroll
            for (int j = 0; j < 3; j++) G.a[i][j] = fc(__ffma2_rn(y, bc2(u[j]), f2(G.a[i][j])));
        }
    }
}

// G = S = 1 + z1 u1 u1^T + z2 u2 u2^T
__device__ __forceinline__ void layer_to_gen(const Layer& f, cg9& G) {
    const float2 z0 = make_float2(f.z[0][0], f.z[0][1]), z1 = make_float2(f.z[1][0], f.z[1][1]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const float2 p0 = bc2(f.u[0][i] * f.u[0][j]), p1 = bc2(f.u[1][i] * f.u[1][j]);
            const float2 v =
                __ffma2_rn(z1, p1, __ffma2_rn(z0, p0, make_float2(i == j ? 1.0f : 0.0f, 0.0f)));
            G.a[i][j] = fc(v);
            G.a[j][i] = fc(v);
        }
}

// Complex dot products over k of 3 with paired FMAs: the products of x's real parts and of
// its imaginary parts with the (re, im) pairs of y accumulate separately, so no lane swap is
// needed; sum_k x_k y_k = (r.x - i.y, r.y + i.x) and sum_k conj(x_k) y_k = (r.x + i.y,
// r.y - i.x) with r = sum re(x_k) y_k, i = sum im(x_k) y_k.
struct cacc {
    float2 r, i;
};
__device__ __forceinline__ cacc cdot3(cf x0, cf y0, cf x1, cf y1, cf x2, cf y2) {
    cacc a;
    a.r = __fmul2_rn(bc2(x0.re), f2(y0));
    a.i = __fmul2_rn(bc2(x0.im), f2(y0));
    a.r = __ffma2_rn(bc2(x1.re), f2(y1), a.r);
    a.i = __ffma2_rn(bc2(x1.im), f2(y1), a.i);
    a.r = __ffma2_rn(bc2(x2.re), f2(y2), a.r);
    a.i = __ffma2_rn(bc2(x2.im), f2(y2), a.i);
    return a;
}

// One Newton-Schulz step toward the nearest unitary matrix, A <- A (3 - A^+ A) / 2.  The
// rounding of FP32 layer matrices leaves each slightly non-unitary and that part of the
// error accumulates over the ~2M products of a deep trajectory; one step at the end removes
// it to second order (measured: max error on the 59-shell, 2000 x 2000 grid drops by ~2x).
// A^+ A is Hermitian: its upper triangle is formed and mirrored.
__device__ __forceinline__ void newton_schulz(cg9& A) {
    cg9 G;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        // diagonal: sum_k |A_ki|^2
        float2 q = __fmul2_rn(f2(A.a[0][i]), f2(A.a[0][i]));
        q = __ffma2_rn(f2(A.a[1][i]), f2(A.a[1][i]), q);
        q = __ffma2_rn(f2(A.a[2][i]), f2(A.a[2][i]), q);
        G.a[i][i] = cf{1.5f - 0.5f * (q.x + q.y), 0.0f};
#pragma unroll
        for (int j = i + 1; j < 3; j++) {
            const cacc h = cdot3(A.a[0][i], A.a[0][j], A.a[1][i], A.a[1][j], A.a[2][i], A.a[2][j]);
            const float re = h.r.x + h.i.y, im = h.r.y - h.i.x;  // (A^+ A)_ij
            G.a[i][j] = cf{-0.5f * re, -0.5f * im};
            G.a[j][i] = cf{-0.5f * re, 0.5f * im};
        }
    }
    cg9 R;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const cacc h = cdot3(A.a[i][0], G.a[0][j], A.a[i][1], G.a[1][j], A.a[i][2], G.a[2][j]);
            R.a[i][j] = cf{h.r.x - h.i.y, h.r.y + h.i.x};
        }
    A = R;
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

// Trajectories crossing at least this many shells get the Newton-Schulz step.  Measured max
// |mixed - FP64| on the 59-shell 2000 x 2000 grid (nu and nubar) with the step from M >= 6 /
// 12 / 20 / never: 2.6e-6 / 5.2e-6 / 5.4e-6 / 9.5e-6, the per-bin kernel 0.186 / 0.184 /
// 0.182 / 0.180 ms; on a PREM-12 grid 1.9e-6 / 3.8e-6 / 3.8e-6 / 3.8e-6, the batched PREM-12
// workload 9.00 / 8.63 / 8.62 / 8.62 ms.  Without the step the error grows with the number
// of FP32 layer applications (unitarity drift: 1.5e-6 at M = 2, 4.4e-6 at M = 12, 9.3e-6 at
// M = 59).
constexpr int kNewtonSchulzMinShells = 6;

struct WParams {
    float c, s, er, ei;
};

CP3_HD WParams wparams(const OscParams& p) {
    return WParams{p.wf[0], p.wf[1], p.wf[2], p.wf[3]};
}

// The nine probabilities of a single constant-density layer (a beam baseline, or an
// atmospheric bin that crosses no shell) from the three-flavour expansion over the matter
// eigenstates k = 0, 1, 2, with U_ak = (W u_k)_a the flavour components of eigenstate k:
//   P(a -> b) = delta_ab + 2 sum_{j>k} [Re c_jk (cos D_jk - 1) + Im c_jk sin D_jk],
//   c_jk = w_j conj(w_k),  w_k = U_bk conj(U_ak),  D_jk = phi_j - phi_k  (phi_0 = 0).
// For a = b, c_jk = m_aj m_ak with m_ak = |U_ak|^2, and there is no sine term.  For a != b
// the w_k sum to zero (unitarity), so Re c_jk = W_l - (W_0 + W_1 + W_2) / 2 with
// W_k = m_ak m_bk and l the third index, and Im c_10 = -Im c_20 = Im c_21 = J_ab, the
// Jarlskog invariant in matter (J for e->mu, mu->tau and tau->e, -J for the reverse).
// The nine moduli and J thus give every coefficient once per (energy, density); a path
// length then costs its two phase factors and about 30 FMAs, where forming
// S = 1 + z1 P1 + z2 P2 and turning it into the flavour basis cost about 110.
struct LayerCoefs {
    float d[3][3];  // flavour a's survival: 2 m_aj m_ak for (j, k) = (1, 0), (2, 0), (2, 1)
    float o[3][3];  // the pairs (e, mu), (mu, tau), (tau, e): 2 Re c_jk for the same (j, k)
    float j2;       // 2 J_{e mu}
};

// u[k-1] = the unit eigenvector of eigenstate k in the rotated basis (k = 1, 2); W = [[1,0,0],
// [0,c,s e],[0,-s,c e]], e = e^{i delta}, so U_ek = u_k0, U_mu,k = c u_k1 + s e u_k2 and
// U_tau,k = -s u_k1 + c e u_k2.
__device__ __forceinline__ LayerCoefs layer_coefficients(const float u[2][3], const WParams& w) {
    // eigenstates 1 and 2 side by side
    const float2 u0 = make_float2(u[0][0], u[1][0]), u1 = make_float2(u[0][1], u[1][1]),
                 u2 = make_float2(u[0][2], u[1][2]);
    const float cc = w.c * w.c, ss = w.s * w.s, cs2 = 2.0f * w.c * w.s;
    const float2 b1 = __fmul2_rn(u1, u1), b2 = __fmul2_rn(u2, u2), x = __fmul2_rn(u1, u2);
    const float2 xr = __fmul2_rn(x, bc2(cs2 * w.er));
    float2 m[3];  // m[a] = (|U_a1|^2, |U_a2|^2)
    m[0] = __fmul2_rn(u0, u0);
    m[1] = __ffma2_rn(bc2(cc), b1, __ffma2_rn(bc2(ss), b2, xr));
    m[2] = __ffma2_rn(bc2(ss), b1, __ffma2_rn(bc2(cc), b2, neg2(xr)));
    float m0[3];  // |U_a0|^2
#pragma unroll
    for (int a = 0; a < 3; a++) m0[a] = 1.0f - m[a].x - m[a].y;
    LayerCoefs k;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float t = 2.0f * m0[a];
        k.d[a][0] = t * m[a].x;
        k.d[a][1] = t * m[a].y;
        k.d[a][2] = 2.0f * m[a].x * m[a].y;
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int a = q, b = q == 2 ? 0 : q + 1;
        const float W0 = m0[a] * m0[b], W1 = m[a].x * m[b].x, W2 = m[a].y * m[b].y;
        const float S = W0 + W1 + W2;
        k.o[q][0] = fmaf(2.0f, W2, -S);
        k.o[q][1] = fmaf(2.0f, W1, -S);
        k.o[q][2] = fmaf(2.0f, W0, -S);
    }
    // J_{e mu} = Im(w_2 conj(w_1)), w_k = U_mu,k u_k0: u_10 u_20 c s sin(delta) (u_11 u_22 - u_12 u_21)
    k.j2 = cs2 * w.ei * (u0.x * u0.y) * fmaf(u1.x, u2.y, -(u2.x * u1.y));
    return k;
}

// The nine probabilities of one path length from the coefficients and the phase factors
// z_k = e^{-i phi_k} - 1 (k = 1, 2); channel a*3+b = P(a -> b) at out[ch * plane].
__device__ __forceinline__ void layer_store(const LayerCoefs& k, float2 zr, float2 zi,
                                            float* __restrict__ out, size_t plane) {
    // cos D - 1 for (1,0), (2,0), (2,1); e^{-i D_21} = (1 + z_2) conj(1 + z_1)
    const float g0 = zr.x, g1 = zr.y, g2 = fmaf(zi.x, zi.y, fmaf(zr.x, zr.y, zr.x + zr.y));
    // sin D_10 - sin D_20 + sin D_21 = Im z_1 Re z_2 - Im z_2 Re z_1
    const float jt = k.j2 * fmaf(zi.x, zr.y, -(zi.y * zr.x));
#pragma unroll
    for (int a = 0; a < 3; a++)
        out[(size_t)(a * 4) * plane] = fmaf(k.d[a][2], g2, fmaf(k.d[a][1], g1, fmaf(k.d[a][0], g0, 1.0f)));
    // (e, mu): channels 1 (e->mu) and 3 (mu->e); (mu, tau): 5 and 7; (tau, e): 6 and 2
    constexpr int fwd[3] = {1, 5, 6}, rev[3] = {3, 7, 2};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const float v = fmaf(k.o[q][2], g2, fmaf(k.o[q][1], g1, k.o[q][0] * g0));
        out[(size_t)fwd[q] * plane] = v + jt;
        out[(size_t)rev[q] * plane] = v - jt;
    }
}

// A bin that crosses no shell: the air layer alone, through the expansion.
__device__ __forceinline__ void store_one_layer(const Layer& F, const WParams& w,
                                                float* __restrict__ out, size_t plane) {
    layer_store(layer_coefficients(F.u, w), make_float2(F.z[0][0], F.z[1][0]),
                make_float2(F.z[0][1], F.z[1][1]), out, plane);
}


// One atmospheric bin over M+1 segments, generic in where each segment's layer comes from:
// seg(l, F) fills F for segment l (0 = air, then shells inwards).
// B <- B^T S_M B for the innermost layer F = S_M (complex symmetric: the upper triangle of
// B^T X, X = S_M B, is formed and mirrored).
__device__ __forceinline__ void close_palindrome(const Layer& F, cg9& B) {
    cg9 X = B, Q;
    apply_left(F, X);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = i; j < 3; j++) {
            const cacc h = cdot3(B.a[0][i], X.a[0][j], B.a[1][i], X.a[1][j], B.a[2][i], X.a[2][j]);
            Q.a[i][j] = cf{h.r.x - h.i.y, h.r.y + h.i.x};
        }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < i; j++) Q.a[i][j] = Q.a[j][i];
    B = Q;
}

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
        close_palindrome(F, G);
    }
}

// One atmospheric bin over M+1 segments, generic in where each segment's layer comes from:
// seg(l, F) fills F for segment l (0 = air, then shells inwards).
template <class SegFn>
__device__ __forceinline__ void atmos_bin_mixed_with(SegFn seg, int M, const WParams& w,
                                                     float* __restrict__ out, size_t plane) {
    Layer F;
    if (M == 0) {
        seg(0, F);
        store_one_layer(F, w, out, plane);
        return;
    }
    cg9 A2;
    chain_mixed(seg, M, A2);
    seg(0, F);
    apply_right(F, A2);  // ... S_0
    // One or two FP32 layer matrices are unitary to ~1e-7 already; the correction pays off
    // from the longer chains on (it removes the drift accumulated over ~2M products).
    if (M >= kNewtonSchulzMinShells) newton_schulz(A2);
    store_probabilities(A2, w.c, w.s, w.er, w.ei, out, plane);
}

// One atmospheric bin from the eigen table: the trajectory's segment lengths are in shared
// memory (s_len[0..M]); segment l's density class is l (0 the air, l shell l-1); tab points
// at this bin's energy column of the table (entry of class c at tab + c * cls_stride);
// probabilities go to out[ch * plane].
//
// kPrefetch: each segment's entry is loaded one layer ahead of its use, so that the L2
// latency of the table overlaps the previous layer's arithmetic (the air segment's entry
// comes last).  Measured: 2 % faster in the batched kernel, whose tables are written in the
// same launch; 1 % slower in the single-grid kernel, which therefore loads on use.
template <int kLoad = kLoadReadOnly, bool kPrefetch = false>
__device__ __forceinline__ void atmos_bin_mixed(const float* __restrict__ tab, size_t cls_stride,
                                                const float2* s_len, int M, const WParams& w,
                                                float* __restrict__ out, size_t plane) {
    auto entry = [&](int l) { return load_table_entry<kLoad>(tab + l * cls_stride); };
    if (!kPrefetch) {
        atmos_bin_mixed_with(
            [&](int l, Layer& F) { layer_from_entry(entry(l), s_len[l], F); }, M, w, out, plane);
        return;
    }
    Layer F;
    if (M == 0) {
        layer_from_entry(entry(0), s_len[0], F);
        store_one_layer(F, w, out, plane);
        return;
    }
    cg9 A2;
    TableEntry e = entry(1), n = entry(M > 1 ? 2 : 0);
    layer_from_entry(e, s_len[1], F);
    layer_to_gen(F, A2);  // B = S_1
    if (M > 1) {
        for (int l = 2; l < M; l++) {
            e = n;
            n = entry(l + 1);
            layer_from_entry(e, s_len[l], F);
            apply_left(F, A2);
        }
        e = n;
        n = entry(0);
        layer_from_entry(e, s_len[M], F);
        close_palindrome(F, A2);
    }
    layer_from_entry(n, s_len[0], F);
    apply_right(F, A2);  // ... S_0
    if (M >= kNewtonSchulzMinShells) newton_schulz(A2);  // as in atmos_bin_mixed_with
    store_probabilities(A2, w.c, w.s, w.er, w.ei, out, plane);
}

// Layer of a segment whose density is its own (quadratic density model): the
// eigen-decomposition is solved for this segment (double-float refined).  The _rates form
// also returns the phase rates (the averaging kernel needs the air layer's).
__device__ __forceinline__ void segment_layer_inline_rates(const OscParams* __restrict__ p,
                                                           double E, double rho_e, float2 L,
                                                           Layer& f, float om[2][2]) {
    rotated_eigen_vectors(p, df_from(E), df_from(rho_e), f.u, om);
    float2 lo, zr, zi;
    const float2 r = reduced_turn2(make_float2(om[0][0], om[1][0]),
                                   make_float2(om[0][1], om[1][1]), L.x, L.y, lo);
    unit_turn_minus_one2(r, lo, zr, zi);
    f.z[0][0] = zr.x;
    f.z[0][1] = zi.x;
    f.z[1][0] = zr.y;
    f.z[1][1] = zi.y;
}
__device__ __forceinline__ void segment_layer_inline(const OscParams* __restrict__ p, double E,
                                                     double rho_e, float2 L, Layer& f) {
    float om[2][2];  // the phase rates omega_k / 2 pi (hi, lo), turns per km
    segment_layer_inline_rates(p, E, rho_e, L, f, om);
}

// One beam energy (E, rho_e as double or float pair): eigen-decomposition (double-float
// refined), the energy's coefficients, then for each baseline L[j] its phase factors and
// the nine probabilities at out + j * baseline_stride + ch * plane.
template <class Real>
__device__ __forceinline__ void beam_bin_mixed(const OscParams* __restrict__ p, const WParams& w,
                                               Real E, Real rho_e, const float2* L, int nL,
                                               float* __restrict__ out, size_t plane,
                                               size_t baseline_stride) {
    float u[2][3], om[2][2];
    rotated_eigen_vectors_fp32(p, E, rho_e, u, om);
    const LayerCoefs k = layer_coefficients(u, w);
    for (int j = 0; j < nL; j++) {
        float2 lo, zr, zi;
        const float2 r = reduced_turn2(make_float2(om[0][0], om[1][0]),
                                       make_float2(om[0][1], om[1][1]), L[j].x, L[j].y, lo);
        unit_turn_minus_one2_hw(r, lo, zr, zi);
        layer_store(k, zr, zi, out + j * baseline_stride, plane);
    }
}

}  // namespace cp3

// Arithmetic policies of the propagation chain.
//
//   Q30  : mixed path.  Amplitudes, eigen-bases and overlaps are Q1.30 fixed
//          point (int32, value = x / 2^30, |x| < 2); each 3-term complex dot
//          product is summed exactly in 64 bits from mul.wide.s32 products
//          (32x32 -> 64 on the FMA-heavy pipe; complex products by Gauss's
//          three multiplications) and is rounded once, down
//          (floor, one funnel shift; the overlap tables alternate in sign from
//          layer to layer so that these one-sided errors do not add up along
//          the chain).  Phases are
//          evaluated in FP32 double-float and turned into Q1.30 cos/sin with
//          a 256-entry table and a short FP32 correction.
//   F64  : plain method.  Everything in FP64.
//
// The chain algorithm (cp3_chain.cuh) is written once against these
// operations, so both paths execute the same sequence of steps.
#pragma once

#include <cstdint>

#include "cp3_check.cuh"
#include "cp3_internal.h"

namespace cp3 {

// ---------------------------------------------------------------- Q1.30 ----
// Every product is one mul.wide (IMAD.WIDE); sums are 64-bit adds and
// rounding takes bits 30..61 with one funnel shift, both on the ALU pipe
// (floor), which keeps the FMA-heavy pipe for the products.
struct Q30 {
    using R = int;
    struct C {
        int re, im;
    };
    // flavour_block's order (cp3_chain.cuh): through G = Y^T D_M Y, which
    // frees Y before X' (no spill at the 64-register cap)
    static constexpr bool kBlockByRows = false;

    static __device__ __forceinline__ long long mul(int a, int b) {
        long long d;
        asm("mul.wide.s32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
        return d;
    }
    // Start of an accumulation that ends in rnd.  Rounding half up needs a
    // 2^29 bias here (a 64-bit add, two ALU instructions per rounding, 176
    // per pair); floor rounding needs none and measured 6 % faster on the
    // 4096^2 grid.  Its one-sided errors are kept from adding up along the
    // chain by the sign alternation of the overlap tables (see prep_overlap_v):
    // max |dP| against the FP64 kernel 1.2e-7 (9.5e-8 rounding half up, 1.9e-7
    // floor without the alternation).
    static __device__ __forceinline__ long long mulb(int a, int b) { return mul(a, b); }
    // floor(acc / 2^30)
    static __device__ __forceinline__ int rnd(long long acc) {
        int r;
        asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\tshf.r.clamp.b32 %0, lo, hi, 30;\n\t}"
            : "=r"(r)
            : "l"(acc));
        return r;
    }

    static __device__ __forceinline__ R one() { return 1 << 30; }
    static __device__ __forceinline__ C cz() { return C{0, 0}; }
    static __device__ __forceinline__ C creal(R x) { return C{x, 0}; }
    static __device__ __forceinline__ C conj(C z) { return C{z.re, -z.im}; }

    // t * z  (real times complex)
    __device__ __forceinline__ C mulRC(R t, C z) const { return C{rnd(mulb(t, z.re)), rnd(mulb(t, z.im))}; }
    // The dot products below form every product with mul.wide and add them
    // in a tree of 64-bit adds and subtracts (ALU pipe), instead of chaining
    // mad.wide.s32 (32x32+64 -> 64): the accumulating form holds the
    // FMA-heavy pipe longer than a plain product, and a six-term dot product
    // measured 11 % faster as a tree in a throughput probe on GB300.
    // Two's-complement sums are exact in any order, so the results are
    // bit-identical to the chained form.

    // z * e where e = (c, s), by Gauss's three products: k1 = c (re + im),
    // re = k1 - im (c + s), im = k1 + re (s - c); c + s and s - c are shared
    // by every rotation with the same phase.  All operands stay below 2 in
    // magnitude (|z|, |e| <= 1), and the integer sums are exact, so the result
    // equals the four-product form bit for bit.
    __device__ __forceinline__ C mulPhase(C z, int c, int s, int /*ns*/) const {
        const long long k1 = mulb(c, z.re + z.im);
        return C{rnd(k1 - mul(z.im, c + s)), rnd(k1 + mul(z.re, s - c))};
    }
    // t0 z0 + t1 z1 + t2 z2
    __device__ __forceinline__ C dotRC(R t0, R t1, R t2, C z0, C z1, C z2) const {
        const long long r = (mulb(t0, z0.re) + mul(t1, z1.re)) + mul(t2, z2.re);
        const long long i = (mulb(t0, z0.im) + mul(t1, z1.im)) + mul(t2, z2.im);
        return C{rnd(r), rnd(i)};
    }
    // a b by Gauss's three products: k1 = b.re (a.re + a.im),
    // k2 = a.re (b.im - b.re), k3 = a.im (b.re + b.im); a b = (k1 - k3) +
    // i (k1 + k2), exactly.  Every operand of the chain's complex products is
    // an entry of a unitary matrix or of a unit vector (|a|, |b| <= 1), so the
    // pre-adds stay below 2 and fit Q1.30.
    static __device__ __forceinline__ void gauss(C a, C b, long long& re, long long& im) {
        const long long k1 = mul(b.re, a.re + a.im);
        re = k1 - mul(a.im, b.re + b.im);
        im = k1 + mul(a.re, b.im - b.re);
    }
    // a0 b0 + a1 b1 + a2 b2 (complex)
    __device__ __forceinline__ C dotCC(C a0, C a1, C a2, C b0, C b1, C b2) const {
        long long r0, i0, r1, i1, r2, i2;
        gauss(a0, b0, r0, i0);
        gauss(a1, b1, r1, i1);
        gauss(a2, b2, r2, i2);
        return C{rnd((r0 + r1) + r2), rnd((i0 + i1) + i2)};
    }
    // conj(a0 b1 - a1 b0): one component of conj(u x v)
    __device__ __forceinline__ C crossConj(C a0, C a1, C b0, C b1) const {
        long long r0, i0, r1, i1;
        gauss(a0, b1, r0, i0);
        gauss(a1, b0, r1, i1);
        return C{rnd(r0 - r1), rnd(i1 - i0)};
    }
    // a b (|a|, |b| <= 1), one rounding
    __device__ __forceinline__ C mulCC(C a, C b) const {
        long long re, im;
        gauss(a, b, re, im);
        return C{rnd(re), rnd(im)};
    }
    // q0 + q1 e^{i psi1} + q2 e^{i psi2} (|q_k| <= 1), the rotations by
    // Gauss's three products as in mulPhase, all summed exactly, one rounding
    __device__ __forceinline__ C phaseSum(C q0, C q1, C q2, int c1, int s1, int c2, int s2) const {
        const long long k1 = mul(c1, q1.re + q1.im), k2 = mul(c2, q2.re + q2.im);
        const long long re = ((long long)q0.re << 30) + (k1 - mul(q1.im, c1 + s1)) + (k2 - mul(q2.im, c2 + s2));
        const long long im = ((long long)q0.im << 30) + (k1 + mul(q1.re, s1 - c1)) + (k2 + mul(q2.re, s2 - c2));
        return C{rnd(re), rnd(im)};
    }
    // |z|^2 exactly, as Q2.60 in 64 bits
    static __device__ __forceinline__ long long norm2(C z) { return mul(z.re, z.re) + mul(z.im, z.im); }
    // Q2.60 probability -> float, one rounding; the completed entries of the
    // doubly stochastic matrix may come out a few 1e-10 below zero: clamp
    static __device__ __forceinline__ float to_prob(long long q) {
        return q <= 0 ? 0.0f : q2_60_to_float(q);
    }
    static __device__ __forceinline__ float q2_60_to_float(long long q) {
        return __ll2float_rn(q) * 8.673617379884035e-19f;  // 2^-60
    }
    // the nine probabilities from the 2x2 block B = (S[e][e], S[e][mu], S[mu][e], S[mu][mu])
    // of a unitary S: out[in*3+out] = |S[out][in]|^2, rows and columns summing to one
    static __device__ __forceinline__ void complete(const C B[4], float out[9]) {
        const long long one = 1LL << 60;
        const long long q00 = norm2(B[0]), q01 = norm2(B[1]), q10 = norm2(B[2]), q11 = norm2(B[3]);
        // q[out][in]
        const long long q02 = one - q00 - q01, q12 = one - q10 - q11;
        const long long q20 = one - q00 - q10, q21 = one - q01 - q11;
        const long long q22 = q00 + q01 + q10 + q11 - one;
        // the four squared moduli are >= 0 and need no clamp (same bits)
        out[0] = q2_60_to_float(q00); out[1] = q2_60_to_float(q10); out[2] = to_prob(q20);
        out[3] = q2_60_to_float(q01); out[4] = q2_60_to_float(q11); out[5] = to_prob(q21);
        out[6] = to_prob(q02); out[7] = to_prob(q12); out[8] = to_prob(q22);
    }
    // averages over production heights: |z|^2 as a float (one rounding of the
    // exact Q2.60 value), weighted sums in FP32, completion of the averaged
    // block (the completion is linear, so averaging commutes with it)
    using Acc = float;
    static __device__ __forceinline__ float prob(C z) { return __ll2float_rn(norm2(z)) * 8.673617379884035e-19f; }
    static __device__ __forceinline__ void complete_avg(float q00, float q01, float q10, float q11, float out[9]) {
        out[0] = q00; out[1] = q10; out[2] = fmaxf(1.0f - q00 - q10, 0.0f);
        out[3] = q01; out[4] = q11; out[5] = fmaxf(1.0f - q01 - q11, 0.0f);
        out[6] = fmaxf(1.0f - q00 - q01, 0.0f); out[7] = fmaxf(1.0f - q10 - q11, 0.0f);
        out[8] = fmaxf((q00 + q01) + (q10 + q11) - 1.0f, 0.0f);
    }
};

// Q1.30 cos/sin of 2*pi*t for a phase t = kappa * L given in turns as two
// double-float factors (kh + kl) * (Lh + Ll).
//   1. t in double-float: p + e with p = kh*Lh rounded and e its exact error
//      plus the cross terms;
//   2. reduce: u = p - rint(p) (exact), j = rint(256 u), d = (u - j/256) + e,
//      so t = integer + j/256 + d with |d| <= 1/512 (+ rounding);
//   3. x = 2 pi d (2 pi as a float: 3.4e-10 rad at most); sin x = x - x^3/6
//      and cos x - 1 = -x^2/2 + x^4/24 in FP32 (truncation below 3e-12 for
//      |x| <= pi/256);
//   4. rotate the table entry (C, S) = (cos, sin)(2 pi j/256) by x: the
//      corrections C (cos x - 1) - S sin x and S (cos x - 1) + C sin x are
//      below 0.013 in magnitude, so FP32 carries them to ~1e-9 absolute, and
//      they are added to the exact Q1.30 table entry.
// `tab` holds 257 entries (Q1.30 cos, Q1.30 sin, float cos * 2^30, float
// sin * 2^30: the corrections come out in Q1.30 units) for j = -128..128 at
// index j + 128.  u lies in [-1/2, 1/2], so j = rint(256 u) is in range; a
// NaN phase converts to j = 0.
// rint(256 u) for |u| <= 1/2 by adding 1.5 * 2^23: the sum's last place is 1,
// so the add rounds to the nearest integer with ties to even (as rintf does),
// and the integer sits in the low bits of the sum's encoding
// (kRoundOffsetBits + j), which also serves as the table index without a
// float-to-int conversion.
constexpr float kRoundOffset = 12582912.0f;  // 1.5 * 2^23
constexpr int kRoundOffsetBits = 0x4B400000;

// Q1.30 cos/sin of 2 pi (p + e) for a phase given in turns as a double-float
// pair (|e| small against 1): steps 2-4 above.  Also returns the encoding of
// the offset sum (jbits, whose low 8 bits are j mod 256) and the remainder d,
// from which the caller can sum phases (TurnSum).
__device__ __forceinline__ void turns_q30_u(float u, float e, const int4* __restrict__ tab, int& cq, int& sq,
                                            int& jbits, float& d) {
    const float t = __fmaf_rn(u, 256.0f, kRoundOffset);
    const float j = __fsub_rn(t, kRoundOffset);
    d = fmaf(j, -0.00390625f, u) + e;
    jbits = __float_as_int(t);
    // sin(2 pi d) and cos(2 pi d) - 1 with 2 pi folded into the coefficients
    const float d2 = d * d;
    const float sx = d * fmaf(d2, -4.134170224e+01f, 6.283185307e+00f);
    const float cm = d2 * fmaf(d2, 6.493939402e+01f, -1.973920880e+01f);
    // index j + 128 in [0, 256]; a NaN phase lands past the end and is held
    // at the last entry (its d is NaN, so the result is NaN either way)
    const unsigned ix = min((unsigned)(jbits - (kRoundOffsetBits - kPhaseTabN / 2)), (unsigned)kPhaseTabN);
    const int4 t4 = tab[CP3_IX(kSitePhaseTable, (int)ix, kPhaseTabN + 1)];
    const float cf = __int_as_float(t4.z), sf = __int_as_float(t4.w);
    const float dc = fmaf(cf, cm, -sf * sx);  // Q1.30 units
    const float ds = fmaf(sf, cm, cf * sx);
    cq = t4.x + __float2int_rn(dc);
    sq = t4.y + __float2int_rn(ds);
}
__device__ __forceinline__ void turns_q30_u(float u, float e, const int4* __restrict__ tab, int& cq, int& sq) {
    int jbits;
    float d;
    turns_q30_u(u, e, tab, cq, sq, jbits, d);
}
__device__ __forceinline__ void turns_q30(float p, float e, const int4* __restrict__ tab, int& cq, int& sq) {
    turns_q30_u(p - rintf(p), e, tab, cq, sq);
}

// t = (kh + kl) (Lh + Ll) turns as p + e: p = kh*Lh rounded, e its exact
// rounding error plus the cross terms (step 1 above).
__device__ __forceinline__ void turns_product(float kh, float kl, float Lh, float Ll, float& p, float& e) {
    p = kh * Lh;
    e = fmaf(kh, Lh, -p);
    e = fmaf(kh, Ll, e);
    e = fmaf(kl, Lh, e);
}

__device__ __forceinline__ void phase_q30(float kh, float kl, float Lh, float Ll, const int4* __restrict__ tab,
                                          int& cq, int& sq) {
    float p, e;
    turns_product(kh, kl, Lh, Ll, p, e);
    turns_q30(p, e, tab, cq, sq);
}

// Running sum of phases in turns as a Q0.32 fixed-point fraction: only
// e^{2 pi i sum} is needed, so the sum is kept modulo one turn by the 32-bit
// wrap-around.  A phase t = integer + j/256 + d (turns_q30_u) adds j exactly
// (as the low 8 bits of its offset encoding, summed apart and moved to bits
// 24..31 at the end) and d rounded to 2^-32 turns.
struct TurnSum {
    unsigned jsum = 0u;  // sum of jbits: low 8 bits are sum(j) mod 256
    unsigned dsum = 0u;  // sum of round(d * 2^32)
    __device__ __forceinline__ void add(int jbits, float d) {
        jsum += (unsigned)jbits;
        dsum += (unsigned)__float2int_rn(d * 4294967296.0f);
    }
    // the sum as a reduced float u in [-1/2, 1/2) and its exact remainder e
    __device__ __forceinline__ void split(float& u, float& e) const {
        const int a = (int)((jsum << 24) + dsum);
        u = (float)a * 2.3283064365386963e-10f;  // 2^-32
        e = (float)(a - __float2int_rn(u * 4294967296.0f)) * 2.3283064365386963e-10f;
    }
};

// ------------------------------------------------------------------ FP64 ----
// max(x, 0) for a double on the integer pipe (sign of the high word).
__device__ __forceinline__ double clamp0(double x) { return (__double2hiint(x) < 0) ? 0.0 : x; }

struct F64 {
    using R = double;
    struct C {
        double re, im;
    };
    // flavour_block's order (cp3_chain.cuh): by rows of Y, 9 products fewer
    static constexpr bool kBlockByRows = true;
    static __device__ __forceinline__ R one() { return 1.0; }
    static __device__ __forceinline__ C cz() { return C{0.0, 0.0}; }
    static __device__ __forceinline__ C creal(R x) { return C{x, 0.0}; }
    static __device__ __forceinline__ C conj(C z) { return C{z.re, -z.im}; }
    static __device__ __forceinline__ C mulRC(R t, C z) { return C{t * z.re, t * z.im}; }
    static __device__ __forceinline__ C mulCC(C a, C b) {
        return C{fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re)};
    }
    // q0 + q1 e^{i psi1} + q2 e^{i psi2}
    static __device__ __forceinline__ C phaseSum(C q0, C q1, C q2, double c1, double s1, double c2, double s2) {
        return C{q0.re + fma(q1.re, c1, -q1.im * s1) + fma(q2.re, c2, -q2.im * s2),
                 q0.im + fma(q1.im, c1, q1.re * s1) + fma(q2.im, c2, q2.re * s2)};
    }
    static __device__ __forceinline__ C mulPhase(C z, double c, double s, double /*ns*/) {
        return C{fma(z.re, c, -z.im * s), fma(z.im, c, z.re * s)};
    }
    static __device__ __forceinline__ C dotRC(R t0, R t1, R t2, C z0, C z1, C z2) {
        return C{fma(t2, z2.re, fma(t1, z1.re, t0 * z0.re)), fma(t2, z2.im, fma(t1, z1.im, t0 * z0.im))};
    }
    static __device__ __forceinline__ C dotCC(C a0, C a1, C a2, C b0, C b1, C b2) {
        double r = a0.re * b0.re;
        r = fma(-a0.im, b0.im, r);
        r = fma(a1.re, b1.re, r);
        r = fma(-a1.im, b1.im, r);
        r = fma(a2.re, b2.re, r);
        r = fma(-a2.im, b2.im, r);
        double i = a0.re * b0.im;
        i = fma(a0.im, b0.re, i);
        i = fma(a1.re, b1.im, i);
        i = fma(a1.im, b1.re, i);
        i = fma(a2.re, b2.im, i);
        i = fma(a2.im, b2.re, i);
        return C{r, i};
    }
    // conj(a0 b1 - a1 b0)
    static __device__ __forceinline__ C crossConj(C a0, C a1, C b0, C b1) {
        const double re = fma(a0.re, b1.re, -a0.im * b1.im) - fma(a1.re, b0.re, -a1.im * b0.im);
        const double im = fma(a0.re, b1.im, a0.im * b1.re) - fma(a1.re, b0.im, a1.im * b0.re);
        return C{re, -im};
    }
    static __device__ __forceinline__ void complete(const C B[4], double out[9]) {
        const double q00 = fma(B[0].re, B[0].re, B[0].im * B[0].im), q01 = fma(B[1].re, B[1].re, B[1].im * B[1].im);
        const double q10 = fma(B[2].re, B[2].re, B[2].im * B[2].im), q11 = fma(B[3].re, B[3].re, B[3].im * B[3].im);
        const double q02 = 1.0 - q00 - q01, q12 = 1.0 - q10 - q11;
        const double q20 = 1.0 - q00 - q10, q21 = 1.0 - q01 - q11;
        const double q22 = q00 + q01 + q10 + q11 - 1.0;
        out[0] = q00; out[1] = q10; out[2] = clamp0(q20);
        out[3] = q01; out[4] = q11; out[5] = clamp0(q21);
        out[6] = clamp0(q02); out[7] = clamp0(q12); out[8] = clamp0(q22);
    }
    using Acc = double;
    static __device__ __forceinline__ double prob(C z) { return fma(z.re, z.re, z.im * z.im); }
    static __device__ __forceinline__ void complete_avg(double q00, double q01, double q10, double q11,
                                                        double out[9]) {
        out[0] = q00; out[1] = q10; out[2] = clamp0(1.0 - q00 - q10);
        out[3] = q01; out[4] = q11; out[5] = clamp0(1.0 - q01 - q11);
        out[6] = clamp0(1.0 - q00 - q01); out[7] = clamp0(1.0 - q10 - q11);
        out[8] = clamp0(q00 + q01 + q10 + q11 - 1.0);
    }
};

// FP64 cos/sin of 2 pi t for t in turns, |t| < 2^40, in two steps.
// reduce_turns_f64: j = round(256 t) from adding 1.5 * 2^52 (the sum's low
// word is j mod 2^32) and the exact remainder d = t - j / 256 (one FMA),
// |d| <= 1/512.  sincos_reduced_f64: with x = 2 pi d, |x| <= pi / 256, the
// Taylor series of sin to x^5 and of cos - 1 to x^6 (truncation below
// 1e-17), written in d with 2 pi folded into the coefficients, rotated onto
// entry (j + 128) mod 256 of the 257-entry table of cos, sin of
// 2 pi (k - 128) / 256.  Fifteen FP64 instructions in all for a given t,
// fourteen for a product kappa * L (reduce_product_f64 below), the table
// index on the integer pipe.
__device__ __forceinline__ void reduce_turns_f64(double t, int& j, double& d) {
    const double magic = 6755399441055744.0;  // 1.5 * 2^52
    const double y = fma(t, 256.0, magic);
    j = __double2loint(y);
    d = fma(y - magic, -0.00390625, t);
}

__device__ __forceinline__ void sincos_reduced_f64(int j, double d, const double2* __restrict__ tab, double& c,
                                                   double& s) {
    // sin(2 pi d) and cos(2 pi d) - 1 with 2 pi folded into the coefficients
    const double d2 = d * d;
    double p = fma(d2, 81.60524927607506, -41.34170224039976);
    p = fma(d2, p, 6.283185307179586);
    const double sx = d * p;
    double q = fma(d2, -85.45681720669373, 64.9393940226683);
    q = fma(d2, q, -19.739208802178716);
    const double cm1 = d2 * q;
    const double2 e = tab[(j + 128) & 255];
    c = fma(-e.y, sx, fma(e.x, cm1, e.x));
    s = fma(e.x, sx, fma(e.y, cm1, e.y));
}

__device__ __forceinline__ void sincos_turns_f64(double t, const double2* __restrict__ tab, double& c,
                                                 double& s) {
    int j;
    double d;
    reduce_turns_f64(t, j, d);
    sincos_reduced_f64(j, d, tab, c, s);
}

// The reduction of a product t = kappa * L without rounding t first: adding
// 1.5 * 2^44 to the fused product rounds it to a multiple of 1/256 (the sum's
// last place), whose count j sits in the sum's low word as above, and
// d = kappa * L - j / 256 comes from a second fused multiply-add with the
// exact -j / 256 = 1.5 * 2^44 - y: three FP64 instructions instead of four,
// and d carries one rounding of itself instead of the rounding of t.
__device__ __forceinline__ void reduce_product_f64(double kappa, double L, int& j, double& d) {
    const double magic = 26388279066624.0;  // 1.5 * 2^44
    const double y = fma(kappa, L, magic);
    j = __double2loint(y);
    d = fma(kappa, L, magic - y);
}

// FP64 cos/sin of 2*pi*t, t = kappa * L turns.
__device__ __forceinline__ void phase_f64(double kappa, double L, const double2* tab, double& c, double& s) {
    int j;
    double d;
    reduce_product_f64(kappa, L, j, d);
    sincos_reduced_f64(j, d, tab, c, s);
}

}  // namespace cp3

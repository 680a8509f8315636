// Arithmetic policies of the propagation chain.
//
//   Q30  : mixed path.  Amplitudes, eigen-bases and overlaps are Q1.30 fixed
//          point (int32, value = x / 2^30, |x| < 2); each 3-term complex dot
//          product accumulates exactly in a 64-bit register with
//          mad.wide.s32 (32x32+64 -> 64, the integer FMA path at half the
//          FP32 rate on GB300) and is rounded once, to 2^-31.  Phases are
//          evaluated in FP32 double-float and turned into Q1.30 cos/sin with
//          a 256-entry table and a short FP32 correction.
//   F64  : plain method.  Everything in FP64.
//
// The chain algorithm (cp3_chain.cuh) is written once against these
// operations, so both paths execute the same sequence of steps.
#pragma once

#include <cstdint>

namespace cp3 {

// ---------------------------------------------------------------- Q1.30 ----
struct Q30 {
    using R = int;
    struct C {
        int re, im;
    };
    static constexpr long long kBias = 1LL << 29;  // round-half-up on >> 30

    static __device__ __forceinline__ long long mad(int a, int b, long long c) {
        long long d;
        asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
        return d;
    }
    static __device__ __forceinline__ int rnd(long long acc) { return (int)(acc >> 30); }

    static __device__ __forceinline__ R one() { return 1 << 30; }
    static __device__ __forceinline__ C cz() { return C{0, 0}; }
    static __device__ __forceinline__ C creal(R x) { return C{x, 0}; }

    // t * z  (real times complex)
    static __device__ __forceinline__ C mulRC(R t, C z) {
        return C{rnd(mad(t, z.re, kBias)), rnd(mad(t, z.im, kBias))};
    }
    // a * b
    static __device__ __forceinline__ C mulCC(C a, C b) {
        long long r = mad(a.re, b.re, kBias);
        r = mad(-a.im, b.im, r);
        long long i = mad(a.re, b.im, kBias);
        i = mad(a.im, b.re, i);
        return C{rnd(r), rnd(i)};
    }
    // z * e where e = (c, s) and ns = -s is supplied to save a negation
    static __device__ __forceinline__ C mulPhase(C z, int c, int s, int ns) {
        long long r = mad(z.re, c, kBias);
        r = mad(z.im, ns, r);
        long long i = mad(z.im, c, kBias);
        i = mad(z.re, s, i);
        return C{rnd(r), rnd(i)};
    }
    // t0 z0 + t1 z1 + t2 z2
    static __device__ __forceinline__ C dotRC(R t0, R t1, R t2, C z0, C z1, C z2) {
        long long r = mad(t0, z0.re, kBias);
        r = mad(t1, z1.re, r);
        r = mad(t2, z2.re, r);
        long long i = mad(t0, z0.im, kBias);
        i = mad(t1, z1.im, i);
        i = mad(t2, z2.im, i);
        return C{rnd(r), rnd(i)};
    }
    // a0 b0 + a1 b1 + a2 b2 (complex)
    static __device__ __forceinline__ C dotCC(C a0, C a1, C a2, C b0, C b1, C b2) {
        long long r = mad(a0.re, b0.re, kBias);
        r = mad(-a0.im, b0.im, r);
        r = mad(a1.re, b1.re, r);
        r = mad(-a1.im, b1.im, r);
        r = mad(a2.re, b2.re, r);
        r = mad(-a2.im, b2.im, r);
        long long i = mad(a0.re, b0.im, kBias);
        i = mad(a0.im, b0.re, i);
        i = mad(a1.re, b1.im, i);
        i = mad(a1.im, b1.re, i);
        i = mad(a2.re, b2.im, i);
        i = mad(a2.im, b2.re, i);
        return C{rnd(r), rnd(i)};
    }
    // c*x + s*y  and  -s*x + c*y  for a real rotation of two complex numbers
    static __device__ __forceinline__ void rot(R c, R s, C& x, C& y) {
        const C nx{rnd(mad(s, y.re, mad(c, x.re, kBias))), rnd(mad(s, y.im, mad(c, x.im, kBias)))};
        const C ny{rnd(mad(c, y.re, mad(-s, x.re, kBias))), rnd(mad(c, y.im, mad(-s, x.im, kBias)))};
        x = nx;
        y = ny;
    }
    static __device__ __forceinline__ float prob(C z) {
        const float a = __int2float_rn(z.re) * (1.0f / 1073741824.0f);
        const float b = __int2float_rn(z.im) * (1.0f / 1073741824.0f);
        return fmaf(a, a, b * b);
    }
};

// Q1.30 cos/sin of 2*pi*t for a phase t = kappa * L given in turns as two
// double-float factors (kh + kl) * (Lh + Ll).
//   1. t in double-float: p + e with p = kh*Lh rounded and e its exact error
//      plus the cross terms;
//   2. reduce: u = p - rint(p) (exact), j = rint(256 u), d = (u - j/256) + e,
//      so t = integer + j/256 + d with |d| <= 1/512 (+ rounding);
//   3. x = 2 pi d; sin x = x - x^3/6 and cos x - 1 = -x^2/2 + x^4/24 in FP32
//      (truncation below 3e-12 for |x| <= pi/256);
//   4. rotate the table entry (cos, sin)(2 pi j/256) by x in Q1.30.
// `tab` holds 257 pairs (Q1.30 cos, sin) for j = -128..128 at index j + 128.
__device__ __forceinline__ void phase_q30(float kh, float kl, float Lh, float Ll,
                                          const int2* __restrict__ tab, int& cq, int& sq) {
    const float p = kh * Lh;
    float e = fmaf(kh, Lh, -p);
    e = fmaf(kh, Ll, e);
    e = fmaf(kl, Lh, e);
    const float u = p - rintf(p);
    float j = rintf(u * 256.0f);
    j = fminf(fmaxf(j, -128.0f), 128.0f);
    const float d = fmaf(j, -0.00390625f, u) + e;
    // 2*pi split as 6.28318548202514648 - 1.74845553e-7 (hi + lo = 2*pi to 2^-48)
    const float x = fmaf(d, 6.28318548202514648f, d * -1.7484555314695172e-07f);
    const float x2 = x * x;
    const float sx = x * fmaf(x2, -0.16666666666666666f, 1.0f);
    const float cm = x2 * fmaf(x2, 0.041666666666666664f, -0.5f);
    const int isx = __float2int_rn(sx * 1073741824.0f);
    const int icm = __float2int_rn(cm * 1073741824.0f);
    const int2 cs = tab[(int)j + 128];
    long long ac = Q30::mad(cs.x, icm, Q30::kBias);
    ac = Q30::mad(-cs.y, isx, ac);
    long long as = Q30::mad(cs.y, icm, Q30::kBias);
    as = Q30::mad(cs.x, isx, as);
    cq = cs.x + Q30::rnd(ac);
    sq = cs.y + Q30::rnd(as);
}

// ------------------------------------------------------------------ FP64 ----
struct F64 {
    using R = double;
    struct C {
        double re, im;
    };
    static __device__ __forceinline__ R one() { return 1.0; }
    static __device__ __forceinline__ C cz() { return C{0.0, 0.0}; }
    static __device__ __forceinline__ C creal(R x) { return C{x, 0.0}; }
    static __device__ __forceinline__ C mulRC(R t, C z) { return C{t * z.re, t * z.im}; }
    static __device__ __forceinline__ C mulCC(C a, C b) {
        return C{fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re)};
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
    static __device__ __forceinline__ void rot(R c, R s, C& x, C& y) {
        const C nx{fma(c, x.re, s * y.re), fma(c, x.im, s * y.im)};
        const C ny{fma(c, y.re, -s * x.re), fma(c, y.im, -s * x.im)};
        x = nx;
        y = ny;
    }
    static __device__ __forceinline__ double prob(C z) { return fma(z.re, z.re, z.im * z.im); }
};

// FP64 cos/sin of 2*pi*t, t = kappa * L turns.
__device__ __forceinline__ void phase_f64(double kappa, double L, double& c, double& s) {
    const double t = kappa * L;
    const double r = t - rint(t);
    sincospi(2.0 * r, &s, &c);
}

}  // namespace cp3

// Double-float ("double-word") arithmetic on the FP32 pipes: a value is the
// unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, good to about
// 2^-48 relative (48 significant bits).  On GB300 a warp's FP64 instruction
// holds its SM sub-partition for about 64 cycles, while FP32 instructions issue
// every cycle on two pipes, so the per-(energy, layer) work of the mixed
// prep (eigen-solves, overlaps, phase rates), whose outputs are Q1.30 words and
// float hi/lo pairs, runs in this arithmetic instead of FP64.
//
// The building blocks are the published error-free transformations (Knuth's
// TwoSum, Dekker's FastTwoSum, TwoProd by one fused multiply-add) and the
// double-word algorithms of Joldes, Muller and Popescu, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic" (ACM TOMS
// 44, 2017): DWPlusDW (their Alg. 6, relative error <= 3u^2), DWTimesFP
// (Alg. 9) and DWTimesDW (Alg. 12, <= 5u^2), u = 2^-24.  Every operation is
// an explicitly rounded intrinsic on the device, so no multiply-add is fused
// behind the algorithms' back; host builds compile with -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstring>

#ifndef CP3_HD
#define CP3_HD __host__ __device__ __forceinline__
#endif

namespace cp3 {

struct DF {
    float hi, lo;
};

CP3_HD float f_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
CP3_HD float f_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
CP3_HD float f_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
CP3_HD float f_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
CP3_HD float f_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
CP3_HD float f_sqrt(float a) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}

// s + e = a + b exactly (Knuth)
CP3_HD DF two_sum(float a, float b) {
    const float s = f_add(a, b);
    const float ap = f_sub(s, b);
    const float bp = f_sub(s, ap);
    return DF{s, f_add(f_sub(a, ap), f_sub(b, bp))};
}
// the same when |a| >= |b| (or a = 0) (Dekker)
CP3_HD DF fast_two_sum(float a, float b) {
    const float s = f_add(a, b);
    return DF{s, f_sub(b, f_sub(s, a))};
}
// p + e = a b exactly
CP3_HD DF two_prod(float a, float b) {
    const float p = f_mul(a, b);
    return DF{p, f_fma(a, b, -p)};
}

CP3_HD DF df_of(float a) { return DF{a, 0.0f}; }
// a double-float pair kept in (or read from) an 8-byte double slot, bit for
// bit (hi in the high word); register moves only on the device
CP3_HD void df_store(double* slot, DF x) {
#ifdef __CUDA_ARCH__
    *slot = __hiloint2double(__float_as_int(x.hi), __float_as_int(x.lo));
#else
    const float w[2] = {x.lo, x.hi};
    memcpy(slot, w, sizeof w);
#endif
}
CP3_HD DF df_read(const double* slot) {
#ifdef __CUDA_ARCH__
    const double d = *slot;
    return DF{__int_as_float(__double2hiint(d)), __int_as_float(__double2loint(d))};
#else
    float w[2];
    memcpy(w, slot, sizeof w);
    return DF{w[1], w[0]};
#endif
}
CP3_HD DF df_neg(DF x) { return DF{-x.hi, -x.lo}; }
CP3_HD double df_to_double(DF x) { return (double)x.hi + (double)x.lo; }

// x + y (DWPlusDW)
CP3_HD DF df_add(DF x, DF y) {
    const DF s = two_sum(x.hi, y.hi);
    const DF t = two_sum(x.lo, y.lo);
    const DF v = fast_two_sum(s.hi, f_add(s.lo, t.hi));
    return fast_two_sum(v.hi, f_add(t.lo, v.lo));
}
CP3_HD DF df_sub(DF x, DF y) { return df_add(x, df_neg(y)); }
// x y (DWTimesDW)
CP3_HD DF df_mul(DF x, DF y) {
    const DF c = two_prod(x.hi, y.hi);
    const float t = f_fma(x.hi, y.lo, f_mul(x.lo, y.lo));
    return fast_two_sum(c.hi, f_add(c.lo, f_fma(x.lo, y.hi, t)));
}
// x y for a float y (DWTimesFP)
CP3_HD DF df_mulf(DF x, float y) {
    const DF c = two_prod(x.hi, y);
    return fast_two_sum(c.hi, f_fma(x.lo, y, c.lo));
}
// x / y: a float quotient, its remainder in double-float and one correction
CP3_HD DF df_div(DF x, DF y) {
    const float q1 = f_div(x.hi, y.hi);
    const DF r = df_sub(x, df_mulf(y, q1));
    const float q2 = f_div(r.hi, y.hi);
    return fast_two_sum(q1, q2);
}
// sqrt(x) for x >= 0: the float root and one Newton correction from the
// double-float residual
CP3_HD DF df_sqrt(DF x) {
    if (!(x.hi > 0.0f)) return DF{0.0f, 0.0f};
    const float s = f_sqrt(x.hi);
    const DF r = df_sub(x, two_prod(s, s));
    return fast_two_sum(s, f_div(r.hi, f_add(s, s)));
}
// 1 / sqrt(x) for x > 0
CP3_HD DF df_rsqrt(DF x) {
    const DF s = df_sqrt(x);
    return df_div(DF{1.0f, 0.0f}, s);
}
// x < y, x == y and |x| >= |y| by the (hi, lo) pairs (normalised values)
CP3_HD bool df_less(DF x, DF y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
CP3_HD bool df_nonzero(DF x) { return x.hi != 0.0f; }
CP3_HD DF df_abs(DF x) { return (x.hi < 0.0f) ? df_neg(x) : x; }
CP3_HD bool df_abs_ge(DF x, DF y) { return !df_less(df_abs(x), df_abs(y)); }

}  // namespace cp3

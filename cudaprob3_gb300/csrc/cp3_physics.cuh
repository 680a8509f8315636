// FP64 per-layer physics shared by every kernel of the propagator:
//   * matter eigenvalues of 2E*H by the trigonometric cubic solution of
//     Barger et al. Eqs. 21-22 (the reference's getMfast, physics.hpp:268-341);
//   * real orthonormal eigenvectors from the Lagrange projectors
//     (H - m_a)(H - m_b)/((m_k - m_a)(m_k - m_b)), Eq. 11 (get_product,
//     physics.hpp:346-431), taken in the real basis of H_r;
//   * trajectory lengths inside each shell (physics.hpp:555-580, 613-618).
#pragma once

#include <cmath>
#include <cstring>

#include "cp3_df.cuh"
#include "cp3_internal.h"

#ifndef CP3_HD
#define CP3_HD __host__ __device__ __forceinline__
#endif

namespace cp3 {

// Eigen-decomposition of the real symmetric 2E*H_r of one layer.
//   m[k]       eigenvalues in eV^2 (order of the trigonometric roots)
//   V[3*i+k]   component i of the unit eigenvector of m[k]; det V = +1
// `rhoye` is rho*Ye in g/cm^3 (the reference passes rho*0.5, physics.hpp:651).
//
// The roots are those of Barger Eqs. 21-22 (physics.hpp:284-324): the cubic
// x^3 + a x^2 + b x + g with the reference's coefficients.  The trigonometric
// angle and its cosines are taken in FP32 (a first guess good to ~1e-7), then
// two FP64 Newton steps on the cubic bring each root to FP64 accuracy; this
// replaces the FP64 acos and cos of the reference and is also accurate where
// acos loses digits (arg near +-1).  Eigenvectors: the largest column of the
// Lagrange projector (H - m_a)(H - m_b) for m_0 and m_1, and v_2 = v_0 x v_1,
// which makes every basis right-handed (the propagation kernels rely on
// det T_l = +1 for T_l = V_{l+1}^T V_l).
//
// On GB300 every warp-wide FP64 instruction holds its SM sub-partition for
// about 64 cycles whatever the number of active lanes (measured: a dependent
// DFMA chain, and four independent ones, cost 64 cycles per instruction; four
// warps on one SM 76 cycles), and FP64 compares, min/max and conversions run
// on the same pipe.  So the solve keeps off that pipe whatever FP32 or the
// integer pipe can do exactly or well enough: the trigonometric first guess
// and every ordering decision are FP32; Newton steps scale by an FP32
// reciprocal of the derivative (the step error is then quadratic plus 1e-7
// times linear, below 1e-20 relative after two steps); quotients use div_nr;
// normalisations use rsqrt; sign and magnitude tests and the conversions to
// Q1.30 and float read the bit patterns on the integer pipe; the branch of the
// projector column is a select, not divergent code.

// Bit pattern of a double.
CP3_HD unsigned long long dbits(double x) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    return u;
#endif
}
// |x| as an integer key: |x| >= |y| iff abs_key(x) >= abs_key(y) (no NaNs).
CP3_HD unsigned long long abs_key(double x) { return dbits(x) & 0x7fffffffffffffffULL; }
CP3_HD bool sign_bit(double x) { return (long long)dbits(x) < 0; }
CP3_HD bool nonzero(double x) { return abs_key(x) != 0; }
// x < y (no NaNs; -0 orders below +0).
CP3_HD bool less_than(double x, double y) {
    const long long a = (long long)dbits(x), b = (long long)dbits(y);
    return (a ^ ((a >> 63) & 0x7fffffffffffffffLL)) < (b ^ ((b >> 63) & 0x7fffffffffffffffLL));
}

// __double2int_rn(x * 2^30) for |x| < 2 from the bits: the significand
// shifted right by 1045 - exponent (at most 63: anything below 2^-31 rounds to
// zero), rounded half to even.  Branch-free.
CP3_HD int q30_rn(double x) {
    const unsigned long long b = dbits(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    const int sh = (1045 - ex < 63) ? 1045 - ex : 63;
    const unsigned long long m = (b & 0xfffffffffffffULL) | (1ULL << 52);
    const unsigned long long r = (m + ((1ULL << (sh - 1)) - 1) + ((m >> sh) & 1)) >> sh;
    return ((long long)b < 0) ? -(int)r : (int)r;
}

// (float)x rounded to nearest even from the bits, branch-free; results below
// FLT_MIN flush to a signed zero (the kernels convert magnitudes far above
// it), overflow gives infinity and NaN stays NaN.
CP3_HD float f32_rn(double x) {
    const unsigned long long b = dbits(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xfffffffffffffULL;
    const unsigned int r = (unsigned int)((m + 0xfffffffULL + ((m >> 29) & 1)) >> 29);  // may carry into the exponent
    unsigned int u = (sign | ((unsigned int)(ex - 1023 + 127) << 23)) + r;
    u = (ex < 1023 - 126) ? sign : u;
    u = (ex > 1023 + 127) ? (sign | 0x7f800000u) : u;
    u = (ex == 0x7ff && m != 0) ? 0x7fc00000u : u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// (double)f from the bits, branch-free and exact for normal floats, zero,
// infinity and NaN; subnormal floats flush to a signed zero.
CP3_HD double f64_of(float f) {
#ifdef __CUDA_ARCH__
    const unsigned int u = __float_as_uint(f);
#else
    unsigned int u;
    std::memcpy(&u, &f, 4);
#endif
    const unsigned int ex = (u >> 23) & 0xff;
    const unsigned int ex64 = (ex == 0xff) ? 0x7ffu : ex + (1023 - 127);
    unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) | ((unsigned long long)ex64 << 52) |
                           ((unsigned long long)(u & 0x7fffffu) << 29);
    b = (ex == 0) ? ((unsigned long long)(u & 0x80000000u) << 32) : b;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

// a / b to about 1 ulp: FP32 reciprocal estimate refined by two Newton-Raphson
// corrections of the quotient, q += r (a - q b) (each squares the relative
// error: 1e-7 -> 1e-14 -> 1e-28).  |b| must lie in FP32's normal range.
CP3_HD double div_nr(double a, double b) {
    const double r = f64_of(1.0f / f32_rn(b));
    double q = a * r;
    q = fma(r, fma(-q, b, a), q);
    q = fma(r, fma(-q, b, a), q);
    return q;
}

CP3_HD double rsqrt_fp64(double x) {
#ifdef __CUDA_ARCH__
    return rsqrt(x);
#else
    return 1.0 / std::sqrt(x);
#endif
}

CP3_HD double cubic_newton(double x, double a, double b, double g) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const double p = fma(fma(x + a, x, b), x, g);
        const double dp = fma(fma(3.0, x, 2.0 * a), x, b);
        x = nonzero(dp) ? x - p * f64_of(1.0f / f32_rn(dp)) : x;
    }
    return x;
}

// Column of N = (H - ma)(H - mb), which is parallel to the eigenvector of the
// third eigenvalue: the column with the largest diagonal entry (H symmetric),
// unnormalised.
CP3_HD void projector_column(const double H[9], double ma, double mb, double c[3]) {
    const double a0 = H[0] - ma, a4 = H[4] - ma, a8 = H[8] - ma;
    const double b0 = H[0] - mb, b4 = H[4] - mb, b8 = H[8] - mb;
    const double n00 = a0 * b0 + H[1] * H[1] + H[2] * H[2];
    const double n11 = H[1] * H[1] + a4 * b4 + H[5] * H[5];
    const double n22 = H[2] * H[2] + H[5] * H[5] + a8 * b8;
    const unsigned long long k0 = abs_key(n00), k1 = abs_key(n11), k2 = abs_key(n22);
    const int p = (k0 >= k1 && k0 >= k2) ? 0 : (k1 >= k2) ? 1 : 2;
    // column p of H - mb, then c = (H - ma) x
    const double x0 = (p == 0) ? b0 : (p == 1) ? H[1] : H[2];
    const double x1 = (p == 1) ? b4 : (p == 0) ? H[1] : H[5];
    const double x2 = (p == 2) ? b8 : (p == 0) ? H[2] : H[5];
    c[0] = a0 * x0 + H[1] * x1 + H[2] * x2;
    c[1] = H[1] * x0 + a4 * x1 + H[5] * x2;
    c[2] = H[2] * x0 + H[5] * x1 + a8 * x2;
}

// Deterministic sign of an eigenvector: its largest component positive.
CP3_HD bool negative_largest(const double c[3]) {
    double big = c[0];
    if (abs_key(c[1]) > abs_key(big)) big = c[1];
    if (abs_key(c[2]) > abs_key(big)) big = c[2];
    return sign_bit(big);
}

CP3_HD void layer_eigen(const OscParams& p, double E, double rhoye, double m[3], double V[9]) {
    // physics.hpp:277-295: matter term and the cubic's coefficients (the
    // parameter-only products are formed once on the host)
    const double fac = p.anti ? kGF * E * rhoye : -(kGF * E * rhoye);
    const double a = fac + p.ca;
    const double b = fma(fac, p.cb1, p.cb0);
    const double g = fac * p.cg;
    // physics.hpp:298-324: trigonometric roots as an FP32 first guess (the
    // numerator and a^2 - 3b are formed in FP64: they cancel), then Newton
    double tmp = a * a - 3.0 * b;
    if (sign_bit(tmp)) tmp = 0.0;
    const float tmpf = f32_rn(tmp);
    const float sqf = sqrtf(tmpf);
    float arg = f32_rn(2.0 * a * a * a - 9.0 * a * b + 27.0 * g) / (2.0f * sqf * tmpf);
    if (!(fabsf(arg) <= 1.0f)) arg = (arg > 0.0f) ? 1.0f : -1.0f;
    const float th = acosf(arg) * (1.0f / 3.0f);
    float sf, cf;
    sincosf(th, &sf, &cf);
    const float hf = 0.866025403784438647f;  // sin(2pi/3)
    const float ampf = -(2.0f / 3.0f) * sqf;
    const float shf = f32_rn(a) * (-1.0f / 3.0f);
    const float q0 = ampf * cf + shf;                     // cos(th)
    const float q1 = ampf * (-0.5f * cf + hf * sf) + shf; // cos(th - 2pi/3)
    const float q2 = ampf * (-0.5f * cf - hf * sf) + shf; // cos(th + 2pi/3)
    // Newton converges fast only on a well separated root, and the degeneracy
    // break leaves a pair 5e-9 eV^2 apart: refine the most isolated root i,
    // then take the other two from the deflated quadratic x^2 - S x + P with
    // S = -a - m_i and P = -g/m_i (or b - m_i S when m_i is not the largest).
    const float d01 = fabsf(q0 - q1), d02 = fabsf(q0 - q2), d12 = fabsf(q1 - q2);
    const float e0 = fminf(d01, d02), e1 = fminf(d01, d12), e2 = fminf(d02, d12);
    const int ri = (e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2) ? 1 : 2;
    const int rj = (ri == 2) ? 0 : ri + 1, rk = (ri == 0) ? 2 : ri - 1;
    const float qi = (ri == 0) ? q0 : (ri == 1) ? q1 : q2;
    const float qj = (rj == 0) ? q0 : (rj == 1) ? q1 : q2;
    const float qk = (rk == 0) ? q0 : (rk == 1) ? q1 : q2;
    const float ej = (rj == 0) ? e0 : (rj == 1) ? e1 : e2;
    const float ek = (rk == 0) ? e0 : (rk == 1) ? e1 : e2;
    const double mi = cubic_newton(f64_of(qi), a, b, g);
    const double S = -a - mi;
    const double P =
        (fabsf(qi) >= fabsf(qj) && fabsf(qi) >= fabsf(qk) && nonzero(mi)) ? div_nr(-g, mi) : b - mi * S;
    double disc = S * S - 4.0 * P;
    if (sign_bit(disc)) disc = 0.0;
    const double big = 0.5 * (S + copysign(sqrt(disc), S));
    const double small = nonzero(big) ? div_nr(P, big) : 0.0;
    const bool big_lo = less_than(big, small);
    const double hi = big_lo ? small : big, lo = big_lo ? big : small;
    const double mj = (qj >= qk) ? hi : lo;
    const double mk = (qj >= qk) ? lo : hi;
    m[0] = (ri == 0) ? mi : (rj == 0) ? mj : mk;
    m[1] = (ri == 1) ? mi : (rj == 1) ? mj : mk;
    m[2] = (ri == 2) ? mi : (rj == 2) ? mj : mk;

    // H_r = O diag(0, d1, d2) O^T - fac e0 e0^T
    const double H[9] = {p.hv[0] - fac, p.hv[1], p.hv[2], p.hv[1], p.hv[3], p.hv[4], p.hv[2], p.hv[4], p.hv[5]};

    // The most isolated eigenvalue i gets its projector column; the next most
    // isolated j too, made exactly orthogonal to v_i; the third is their cross
    // product.  A near-degenerate pair (the degeneracy break of
    // propagator.hpp:226-248) then still yields an orthonormal basis.  The
    // ranking is the FP32 one of the first guesses.
    const bool cyc = ej >= ek;  // j = i+1, k = i+2 (cyclic) or j = i+2, k = i+1
    const int i = ri, j = cyc ? rj : rk;
    const double mje = cyc ? mj : mk, mke = cyc ? mk : mj;
    // v_i normalised; v_j's column orthogonalised against v_i before its one
    // normalisation (the sign of each from its column's largest component)
    double vi[3], vj[3], vk[3];
    projector_column(H, mje, mke, vi);
    projector_column(H, mke, mi, vj);
    {
        const double n2 = vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
        double inv = nonzero(n2) ? rsqrt_fp64(n2) : 0.0;
        if (negative_largest(vi)) inv = -inv;
        vi[0] *= inv;
        vi[1] *= inv;
        vi[2] *= inv;
    }
    const bool neg_j = negative_largest(vj);
    const double d = vj[0] * vi[0] + vj[1] * vi[1] + vj[2] * vi[2];
    vj[0] -= d * vi[0];
    vj[1] -= d * vi[1];
    vj[2] -= d * vi[2];
    const double nj2 = vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2];
    double rj2 = nonzero(nj2) ? rsqrt_fp64(nj2) : 0.0;
    if (neg_j) rj2 = -rj2;
    vj[0] *= rj2;
    vj[1] *= rj2;
    vj[2] *= rj2;
    // (i, j, k) cyclic: v_k = v_i x v_j; otherwise v_k = v_j x v_i
    const double sgn = cyc ? 1.0 : -1.0;
    vk[0] = sgn * (vi[1] * vj[2] - vi[2] * vj[1]);
    vk[1] = sgn * (vi[2] * vj[0] - vi[0] * vj[2]);
    vk[2] = sgn * (vi[0] * vj[1] - vi[1] * vj[0]);
#pragma unroll
    for (int r = 0; r < 3; r++) {
#pragma unroll
        for (int c = 0; c < 3; c++) V[3 * r + c] = (c == i) ? vi[r] : (c == j) ? vj[r] : vk[r];
    }
}

// Phase rate factor of the layer propagator: eigenvalue k's phase relative to
// eigenvalue 0 is -LoEfac * (m_k - m_0) * L / E (physics.hpp:461-467) with the
// per-layer common phase of m_0 removed; in turns per km that is
// phase_rate_factor(E) * (m_k - m_0), the factor computed once per (energy, layer).
CP3_HD double phase_rate_factor(double E) { return div_nr(-kLoEfac / kTwoPi, E); }

// ------------------------------------------------ double-float eigen-solve --
// layer_eigen in double-float arithmetic (cp3_df.cuh) for the mixed prep,
// whose outputs are Q1.30 words and float hi/lo pairs: the same steps (the
// FP32 trigonometric first guess, Newton on the most isolated root,
// deflation, projector columns of the two most isolated roots, the third
// vector as their cross product), on the FP32 pipes instead of FP64.

// double-float split of a double (one FP64 subtraction)
CP3_HD DF df_from_double(double x) {
    const float h = f32_rn(x);
    return DF{h, f32_rn(x - f64_of(h))};
}
CP3_HD DF df_load(const float p[2]) { return DF{p[0], p[1]}; }

constexpr float kGF_hi = (float)kGF;
constexpr float kGF_lo = (float)(kGF - (double)(float)kGF);
constexpr double kRate = -kLoEfac / kTwoPi;  // phase_rate_factor(E) * E
constexpr float kRate_hi = (float)kRate;
constexpr float kRate_lo = (float)(kRate - (double)(float)kRate);

CP3_HD DF df_rate_factor(DF E) { return df_div(DF{kRate_hi, kRate_lo}, E); }

CP3_HD DF cubic_newton_df(DF x, DF a, DF b, DF g) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
        // p(x) = ((x + a) x + b) x + g in double-float; p'(x) in FP32 (the
        // step's error is then quadratic plus 1e-7 times linear)
        const DF p = df_add(df_mul(df_add(df_mul(df_add(x, a), x), b), x), g);
        const float dp = f_fma(f_fma(3.0f, x.hi, f_add(a.hi, a.hi)), x.hi, b.hi);
        if (dp != 0.0f) x = df_sub(x, df_mulf(p, f_div(1.0f, dp)));
    }
    return x;
}

// column of (H - ma)(H - mb) with the largest diagonal entry (projector_column)
CP3_HD void projector_column_df(const DF H[9], DF ma, DF mb, DF c[3]) {
    const DF a0 = df_sub(H[0], ma), a4 = df_sub(H[4], ma), a8 = df_sub(H[8], ma);
    const DF b0 = df_sub(H[0], mb), b4 = df_sub(H[4], mb), b8 = df_sub(H[8], mb);
    // the choice of column only needs the magnitudes: FP32
    const float h1 = H[1].hi, h2 = H[2].hi, h5 = H[5].hi;
    const float n00 = fabsf(f_fma(a0.hi, b0.hi, f_fma(h1, h1, f_mul(h2, h2))));
    const float n11 = fabsf(f_fma(a4.hi, b4.hi, f_fma(h1, h1, f_mul(h5, h5))));
    const float n22 = fabsf(f_fma(a8.hi, b8.hi, f_fma(h2, h2, f_mul(h5, h5))));
    const int p = (n00 >= n11 && n00 >= n22) ? 0 : (n11 >= n22) ? 1 : 2;
    const DF x0 = (p == 0) ? b0 : (p == 1) ? H[1] : H[2];
    const DF x1 = (p == 1) ? b4 : (p == 0) ? H[1] : H[5];
    const DF x2 = (p == 2) ? b8 : (p == 0) ? H[2] : H[5];
    c[0] = df_add(df_add(df_mul(a0, x0), df_mul(H[1], x1)), df_mul(H[2], x2));
    c[1] = df_add(df_add(df_mul(H[1], x0), df_mul(a4, x1)), df_mul(H[5], x2));
    c[2] = df_add(df_add(df_mul(H[2], x0), df_mul(H[5], x1)), df_mul(a8, x2));
}

CP3_HD bool negative_largest_df(const DF c[3]) {
    float big = c[0].hi;
    if (fabsf(c[1].hi) > fabsf(big)) big = c[1].hi;
    if (fabsf(c[2].hi) > fabsf(big)) big = c[2].hi;
    return big < 0.0f;
}

CP3_HD DF df_dot3(const DF x[3], const DF y[3]) {
    return df_add(df_add(df_mul(x[0], y[0]), df_mul(x[1], y[1])), df_mul(x[2], y[2]));
}

CP3_HD void layer_eigen_df(const OscParams& p, DF E, DF rhoye, DF m[3], DF V[9]) {
    // matter term and the cubic's coefficients (physics.hpp:277-295)
    DF fac = df_mul(df_mul(DF{kGF_hi, kGF_lo}, E), rhoye);
    if (!p.anti) fac = df_neg(fac);
    const DF a = df_add(fac, df_load(p.ca_f));
    const DF b = df_add(df_mul(fac, df_load(p.cb1_f)), df_load(p.cb0_f));
    const DF g = df_mul(fac, df_load(p.cg_f));
    // physics.hpp:298-324: FP32 first guess of the trigonometric roots (a^2 - 3b
    // and the numerator cancel: formed in double-float), then Newton
    const DF a2 = df_mul(a, a);
    DF tmp = df_sub(a2, df_mulf(b, 3.0f));
    if (tmp.hi < 0.0f) tmp = DF{0.0f, 0.0f};
    const float tmpf = tmp.hi;
    const float sqf = f_sqrt(tmpf);
    const DF num = df_add(df_sub(df_mulf(df_mul(a2, a), 2.0f), df_mulf(df_mul(a, b), 9.0f)), df_mulf(g, 27.0f));
    float arg = num.hi / (2.0f * sqf * tmpf);
    if (!(fabsf(arg) <= 1.0f)) arg = (arg > 0.0f) ? 1.0f : -1.0f;
    const float th = acosf(arg) * (1.0f / 3.0f);
    float sf, cf;
#ifdef __CUDA_ARCH__
    sincosf(th, &sf, &cf);
#else
    sf = std::sin(th);
    cf = std::cos(th);
#endif
    const float hf = 0.866025403784438647f;  // sin(2pi/3)
    const float ampf = -(2.0f / 3.0f) * sqf;
    const float shf = a.hi * (-1.0f / 3.0f);
    const float q0 = ampf * cf + shf;
    const float q1 = ampf * (-0.5f * cf + hf * sf) + shf;
    const float q2 = ampf * (-0.5f * cf - hf * sf) + shf;
    // refine the most isolated root, deflate for the other two (layer_eigen)
    const float d01 = fabsf(q0 - q1), d02 = fabsf(q0 - q2), d12 = fabsf(q1 - q2);
    const float e0 = fminf(d01, d02), e1 = fminf(d01, d12), e2 = fminf(d02, d12);
    const int ri = (e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2) ? 1 : 2;
    const int rj = (ri == 2) ? 0 : ri + 1, rk = (ri == 0) ? 2 : ri - 1;
    const float qi = (ri == 0) ? q0 : (ri == 1) ? q1 : q2;
    const float qj = (rj == 0) ? q0 : (rj == 1) ? q1 : q2;
    const float qk = (rk == 0) ? q0 : (rk == 1) ? q1 : q2;
    const float ej = (rj == 0) ? e0 : (rj == 1) ? e1 : e2;
    const float ek = (rk == 0) ? e0 : (rk == 1) ? e1 : e2;
    const DF mi = cubic_newton_df(DF{qi, 0.0f}, a, b, g);
    const DF S = df_neg(df_add(a, mi));
    const DF P = (fabsf(qi) >= fabsf(qj) && fabsf(qi) >= fabsf(qk) && df_nonzero(mi)) ? df_neg(df_div(g, mi))
                                                                                       : df_sub(b, df_mul(mi, S));
    DF disc = df_sub(df_mul(S, S), df_mulf(P, 4.0f));
    if (disc.hi < 0.0f) disc = DF{0.0f, 0.0f};
    const DF root = df_sqrt(disc);
    const DF big = df_mulf(df_add(S, (S.hi < 0.0f) ? df_neg(root) : root), 0.5f);
    const DF small = df_nonzero(big) ? df_div(P, big) : DF{0.0f, 0.0f};
    const bool big_lo = df_less(big, small);
    const DF hi = big_lo ? small : big, lo = big_lo ? big : small;
    const DF mj = (qj >= qk) ? hi : lo;
    const DF mk = (qj >= qk) ? lo : hi;
    m[0] = (ri == 0) ? mi : (rj == 0) ? mj : mk;
    m[1] = (ri == 1) ? mi : (rj == 1) ? mj : mk;
    m[2] = (ri == 2) ? mi : (rj == 2) ? mj : mk;

    // H_r = O diag(0, d1, d2) O^T - fac e0 e0^T
    const DF hv0 = df_load(p.hv_f[0]), hv1 = df_load(p.hv_f[1]), hv2 = df_load(p.hv_f[2]);
    const DF hv3 = df_load(p.hv_f[3]), hv4 = df_load(p.hv_f[4]), hv5 = df_load(p.hv_f[5]);
    const DF H[9] = {df_sub(hv0, fac), hv1, hv2, hv1, hv3, hv4, hv2, hv4, hv5};
    const bool cyc = ej >= ek;
    const int i = ri, j = cyc ? rj : rk;
    const DF mje = cyc ? mj : mk, mke = cyc ? mk : mj;
    DF vi[3], vj[3], vk[3];
    projector_column_df(H, mje, mke, vi);
    projector_column_df(H, mke, mi, vj);
    {
        const DF n2 = df_dot3(vi, vi);
        DF inv = df_nonzero(n2) ? df_rsqrt(n2) : DF{0.0f, 0.0f};
        if (negative_largest_df(vi)) inv = df_neg(inv);
#pragma unroll
        for (int r = 0; r < 3; r++) vi[r] = df_mul(vi[r], inv);
    }
    const bool neg_j = negative_largest_df(vj);
    const DF d = df_dot3(vj, vi);
#pragma unroll
    for (int r = 0; r < 3; r++) vj[r] = df_sub(vj[r], df_mul(d, vi[r]));
    {
        const DF n2 = df_dot3(vj, vj);
        DF inv = df_nonzero(n2) ? df_rsqrt(n2) : DF{0.0f, 0.0f};
        if (neg_j) inv = df_neg(inv);
#pragma unroll
        for (int r = 0; r < 3; r++) vj[r] = df_mul(vj[r], inv);
    }
    // (i, j, k) cyclic: v_k = v_i x v_j; otherwise v_k = v_j x v_i
    vk[0] = df_sub(df_mul(vi[1], vj[2]), df_mul(vi[2], vj[1]));
    vk[1] = df_sub(df_mul(vi[2], vj[0]), df_mul(vi[0], vj[2]));
    vk[2] = df_sub(df_mul(vi[0], vj[1]), df_mul(vi[1], vj[0]));
    if (!cyc)
#pragma unroll
        for (int r = 0; r < 3; r++) vk[r] = df_neg(vk[r]);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) V[3 * r + c] = (c == i) ? vi[r] : (c == j) ? vj[r] : vk[r];
}

// round((x.hi + x.lo) 2^30) for |x| < 2: the scaled high part is rounded
// exactly in FP32, the rest added as a small float
CP3_HD int q30_df(DF x) {
    const float h = f_mul(x.hi, 1073741824.0f);
    const float rh = rintf(h);
    const float r = f_add(f_sub(h, rh), f_mul(x.lo, 1073741824.0f));
    return (int)rh + (int)rintf(r);
}

// Products and differences rounded one at a time, as the reference's host
// build evaluates the trajectory geometry (no fused multiply-add): near a
// shell's tangent the chord's square root amplifies a one-ulp difference in
// its argument (cosines one ulp from a shell boundary gave 1e-8 in P from
// contracted products), so the lengths follow the reference's roundings.
// Host builds of these helpers compile with -ffp-contract=off.
CP3_HD double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CP3_HD double sub_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

// Total path length including the production height (physics.hpp:615-616), cm.
CP3_HD double path_length_cm(double c, double height_cm) {
    const double re = kREarth * kKm2Cm;
    const double rh = re + height_cm;
    return sub_rn(sqrt(sub_rn(mul_rn(rh, rh), mul_rn(re * re, sub_rn(1.0, mul_rn(c, c))))), mul_rn(re, c));
}

// Length in km of the segment of layer `l` (0 = atmosphere, 1..M shells from
// the outside in) crossed by a trajectory of cosine c that reaches shell M:
// physics.hpp:555-580 evaluated for the inbound half, l <= M.
// x / 1e5 (cm to km): the product with the rounded reciprocal and one FMA
// correction from the exact remainder, instead of an FP64 division.
CP3_HD double km_of_cm(double x) {
    const double q = x * 1.0e-5;
    return fma(fma(-q, kKm2Cm, x), 1.0e-5, q);
}

CP3_HD double layer_length_km(const double* radii, int l, int M, double c, double path_cm) {
    if (c >= 0.0) return km_of_cm(path_cm);
    const double earth_cm = mul_rn(-2.0 * c, kREarth * kKm2Cm);
    if (l == 0) return km_of_cm(sub_rn(path_cm, earth_cm));
    const int i = l - 1;
    const double perp2 = mul_rn(kREarth * kREarth, sub_rn(1.0, mul_rn(c, c)));
    double q = sub_rn(mul_rn(radii[i], radii[i]), perp2);
    const double cross_this = 2.0 * sqrt(q > 0.0 ? q : 0.0);
    if (i < M - 1) {
        double qn = sub_rn(mul_rn(radii[i + 1], radii[i + 1]), perp2);
        const double cross_next = 2.0 * sqrt(qn > 0.0 ? qn : 0.0);
        return km_of_cm(0.5 * (cross_this - cross_next) * kKm2Cm);
    }
    return km_of_cm(cross_this * kKm2Cm);
}

}  // namespace cp3

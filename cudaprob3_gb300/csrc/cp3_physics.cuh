// FP64 per-layer physics shared by every kernel of the propagator:
//   * matter eigenvalues of 2E*H by the trigonometric cubic solution of
//     Barger et al. Eqs. 21-22 (the reference's getMfast, physics.hpp:268-341);
//   * real orthonormal eigenvectors from the Lagrange projectors
//     (H - m_a)(H - m_b)/((m_k - m_a)(m_k - m_b)), Eq. 11 (get_product,
//     physics.hpp:346-431), taken in the real basis of H_r;
//   * trajectory lengths inside each shell (physics.hpp:555-580, 613-618).
#pragma once

#include <cmath>

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
// FP64 divisions and square roots are long instruction sequences on GB300's
// narrow FP64 pipe, so the solve avoids them where FP32 or a refinement
// suffices: the trigonometric first guess is FP32 throughout; Newton steps
// scale by an FP32 reciprocal of the derivative (the step error is then
// quadratic plus 1e-7 times linear, below 1e-20 relative after two steps);
// quotients use div_nr; normalisations use rsqrt.

// a / b to about 1 ulp: FP32 reciprocal estimate refined by two Newton-Raphson
// corrections of the quotient, q += r (a - q b) (each squares the relative
// error: 1e-7 -> 1e-14 -> 1e-28).  |b| must lie in FP32's normal range.
CP3_HD double div_nr(double a, double b) {
    const double r = (double)(1.0f / (float)b);
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
        if (dp != 0.0) x -= p * (double)(1.0f / (float)dp);
    }
    return x;
}

CP3_HD void eigvec_of(const double H[9], double m, double ma, double mb, double v[3]) {
    // columns of N = (H - ma)(H - mb) are parallel to the eigenvector of m;
    // take the one with the largest diagonal entry
    const double a0 = H[0] - ma, a4 = H[4] - ma, a8 = H[8] - ma;
    const double b0 = H[0] - mb, b4 = H[4] - mb, b8 = H[8] - mb;
    const double n00 = a0 * b0 + H[1] * H[3] + H[2] * H[6];
    const double n11 = H[3] * H[1] + a4 * b4 + H[5] * H[7];
    const double n22 = H[6] * H[2] + H[7] * H[5] + a8 * b8;
    double c0, c1, c2;
    if (fabs(n00) >= fabs(n11) && fabs(n00) >= fabs(n22)) {
        c0 = n00;
        c1 = H[3] * b0 + a4 * H[3] + H[5] * H[6];
        c2 = H[6] * b0 + H[7] * H[3] + a8 * H[6];
    } else if (fabs(n11) >= fabs(n22)) {
        c0 = a0 * H[1] + H[1] * b4 + H[2] * H[7];
        c1 = n11;
        c2 = H[6] * H[1] + H[7] * b4 + a8 * H[7];
    } else {
        c0 = a0 * H[2] + H[1] * H[5] + H[2] * b8;
        c1 = H[3] * H[2] + a4 * H[5] + H[5] * b8;
        c2 = n22;
    }
    const double n2 = c0 * c0 + c1 * c1 + c2 * c2;
    double inv = (n2 > 0.0) ? rsqrt_fp64(n2) : 0.0;
    // deterministic sign: largest component positive
    double big = c0;
    if (fabs(c1) > fabs(big)) big = c1;
    if (fabs(c2) > fabs(big)) big = c2;
    if (big < 0.0) inv = -inv;
    v[0] = c0 * inv;
    v[1] = c1 * inv;
    v[2] = c2 * inv;
}

CP3_HD void layer_eigen(const OscParams& p, double E, double rhoye, double m[3], double V[9]) {
    // physics.hpp:277-295: matter term and the cubic's coefficients
    const double fac = p.anti ? kGF * E * rhoye : -(kGF * E * rhoye);
    const double a = fac + p.dm01 + p.dm02;
    const double b = p.dm01 * p.dm02 + fac * (p.dm01 * (1.0 - p.u01) + p.dm02 * (1.0 - p.u02));
    const double g = fac * p.dm01 * p.dm02 * p.u00;
    // physics.hpp:298-324: trigonometric roots as an FP32 first guess (the
    // numerator and a^2 - 3b are formed in FP64: they cancel), then Newton
    double tmp = a * a - 3.0 * b;
    if (tmp < 0.0) tmp = 0.0;
    const float tmpf = (float)tmp;
    const float sqf = sqrtf(tmpf);
    float arg = (float)(2.0 * a * a * a - 9.0 * a * b + 27.0 * g) / (2.0f * sqf * tmpf);
    if (!(fabsf(arg) <= 1.0f)) arg = (arg > 0.0f) ? 1.0f : -1.0f;
    const float th = acosf(arg) * (1.0f / 3.0f);
    float sf, cf;
    sincosf(th, &sf, &cf);
    const double c = cf, s = sf;
    const double h = 0.86602540378443864676;  // sin(2pi/3)
    const double amp = -(2.0 / 3.0) * (double)sqf;
    const double sh = a * (-1.0 / 3.0);
    {
    double q[3];
    q[0] = amp * c + sh;                   // cos(th)
    q[1] = amp * (-0.5 * c + h * s) + sh;  // cos(th - 2pi/3)
    q[2] = amp * (-0.5 * c - h * s) + sh;  // cos(th + 2pi/3)
    // Newton converges fast only on a well separated root, and the degeneracy
    // break leaves a pair 5e-9 eV^2 apart: refine the most isolated root i,
    // then take the other two from the deflated quadratic x^2 - S x + P with
    // S = -a - m_i and P = -g/m_i (or b - m_i S when m_i is not the largest).
    const double e0 = fmin(fabs(q[0] - q[1]), fabs(q[0] - q[2]));
    const double e1 = fmin(fabs(q[1] - q[0]), fabs(q[1] - q[2]));
    const double e2 = fmin(fabs(q[2] - q[0]), fabs(q[2] - q[1]));
    const int ri = (e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2) ? 1 : 2;
    const int rj = (ri + 1) % 3, rk = (ri + 2) % 3;
    const double qi = (ri == 0) ? q[0] : (ri == 1) ? q[1] : q[2];
    const double qj = (rj == 0) ? q[0] : (rj == 1) ? q[1] : q[2];
    const double qk = (rk == 0) ? q[0] : (rk == 1) ? q[1] : q[2];
    const double mi = cubic_newton(qi, a, b, g);
    const double S = -a - mi;
    const double P = (fabs(mi) >= fabs(qj) && fabs(mi) >= fabs(qk) && mi != 0.0) ? div_nr(-g, mi) : b - mi * S;
    double disc = S * S - 4.0 * P;
    if (disc < 0.0) disc = 0.0;
    const double big = 0.5 * (S + copysign(sqrt(disc), S));
    const double small = (big != 0.0) ? div_nr(P, big) : 0.0;
    const double hi = fmax(big, small), lo = fmin(big, small);
    const double mj = (qj >= qk) ? hi : lo;
    const double mk = (qj >= qk) ? lo : hi;
    m[0] = (ri == 0) ? mi : (rj == 0) ? mj : mk;
    m[1] = (ri == 1) ? mi : (rj == 1) ? mj : mk;
    m[2] = (ri == 2) ? mi : (rj == 2) ? mj : mk;
    }

    // H_r = O diag(0, d1, d2) O^T - fac e0 e0^T
    double H[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            H[3 * i + j] = p.d1 * p.o[3 * i + 1] * p.o[3 * j + 1] + p.d2 * p.o[3 * i + 2] * p.o[3 * j + 2];
    H[0] -= fac;

    // The most isolated eigenvalue i gets its projector column; the next most
    // isolated j too, made exactly orthogonal to v_i; the third is their cross
    // product.  A near-degenerate pair (the degeneracy break of
    // propagator.hpp:226-248) then still yields an orthonormal basis.
    const double g0 = fmin(fabs(m[0] - m[1]), fabs(m[0] - m[2]));
    const double g1 = fmin(fabs(m[1] - m[0]), fabs(m[1] - m[2]));
    const double g2 = fmin(fabs(m[2] - m[0]), fabs(m[2] - m[1]));
    int i = 0;
    if (g1 > g0) i = 1;
    if (g2 > (i == 0 ? g0 : g1)) i = 2;
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    const double gi1 = (i1 == 0) ? g0 : (i1 == 1) ? g1 : g2;
    const double gi2 = (i2 == 0) ? g0 : (i2 == 1) ? g1 : g2;
    const bool cyc = gi1 >= gi2;  // j = i+1, k = i+2 (cyclic) or j = i+2, k = i+1
    const int j = cyc ? i1 : i2;
    const double mi = (i == 0) ? m[0] : (i == 1) ? m[1] : m[2];
    const double mj = (j == 0) ? m[0] : (j == 1) ? m[1] : m[2];
    const int k = 3 - i - j;
    const double mk = (k == 0) ? m[0] : (k == 1) ? m[1] : m[2];
    double vi[3], vj[3], vk[3];
    eigvec_of(H, mi, mj, mk, vi);
    eigvec_of(H, mj, mk, mi, vj);
    const double d = vj[0] * vi[0] + vj[1] * vi[1] + vj[2] * vi[2];
    vj[0] -= d * vi[0];
    vj[1] -= d * vi[1];
    vj[2] -= d * vi[2];
    const double nj2 = vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2];
    const double rj = (nj2 > 0.0) ? rsqrt_fp64(nj2) : 0.0;
    vj[0] *= rj;
    vj[1] *= rj;
    vj[2] *= rj;
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
CP3_HD double phase_rate_factor(double E) { return -kLoEfac / (kTwoPi * E); }

// Total path length including the production height (physics.hpp:615-616), cm.
CP3_HD double path_length_cm(double c, double height_cm) {
    const double re = kREarth * kKm2Cm;
    return sqrt((re + height_cm) * (re + height_cm) - (re * re) * (1.0 - c * c)) - re * c;
}

// Length in km of the segment of layer `l` (0 = atmosphere, 1..M shells from
// the outside in) crossed by a trajectory of cosine c that reaches shell M:
// physics.hpp:555-580 evaluated for the inbound half, l <= M.
CP3_HD double layer_length_km(const double* radii, int l, int M, double c, double path_cm) {
    if (c >= 0.0) return path_cm / kKm2Cm;
    const double earth_cm = -2.0 * c * (kREarth * kKm2Cm);
    if (l == 0) return (path_cm - earth_cm) / kKm2Cm;
    const int i = l - 1;
    const double perp2 = kREarth * kREarth * (1.0 - c * c);
    double q = radii[i] * radii[i] - perp2;
    const double cross_this = 2.0 * sqrt(q > 0.0 ? q : 0.0);
    if (i < M - 1) {
        double qn = radii[i + 1] * radii[i + 1] - perp2;
        const double cross_next = 2.0 * sqrt(qn > 0.0 ? qn : 0.0);
        return (0.5 * (cross_this - cross_next) * kKm2Cm) / kKm2Cm;
    }
    return (cross_this * kKm2Cm) / kKm2Cm;
}

}  // namespace cp3

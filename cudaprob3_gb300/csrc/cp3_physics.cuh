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
//   V[3*i+k]   component i of the unit eigenvector of m[k]
// `rhoye` is rho*Ye in g/cm^3 (the reference passes rho*0.5, physics.hpp:651).
CP3_HD void layer_eigen(const OscParams& p, double E, double rhoye, double m[3], double V[9]) {
    // physics.hpp:277-295: matter term and the cubic's coefficients
    const double fac = p.anti ? kGF * E * rhoye : -(kGF * E * rhoye);
    const double a = fac + p.dm01 + p.dm02;
    const double b = p.dm01 * p.dm02 + fac * (p.dm01 * (1.0 - p.u01) + p.dm02 * (1.0 - p.u02));
    const double g = fac * p.dm01 * p.dm02 * p.u00;
    // physics.hpp:298-324: trigonometric roots
    double tmp = a * a - 3.0 * b;
    if (tmp < 0.0) tmp = 0.0;
    const double sq = sqrt(tmp);
    double arg = (2.0 * a * a * a - 9.0 * a * b + 27.0 * g) / (2.0 * sq * tmp);
    if (!(fabs(arg) <= 1.0)) arg = (arg > 0.0) ? 1.0 : -1.0;
    const double th = acos(arg) / 3.0;
    double s, c;
    sincos(th, &s, &c);
    const double h = 0.86602540378443864676;  // sin(2pi/3)
    const double amp = -(2.0 / 3.0) * sq;
    const double sh = -a / 3.0;
    m[0] = amp * c + sh;                       // cos(th)
    m[1] = amp * (-0.5 * c + h * s) + sh;      // cos(th - 2pi/3)
    m[2] = amp * (-0.5 * c - h * s) + sh;      // cos(th + 2pi/3)

    // H_r = O diag(0, d1, d2) O^T - fac e0 e0^T
    double H[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            H[3 * i + j] = p.d1 * p.o[3 * i + 1] * p.o[3 * j + 1] + p.d2 * p.o[3 * i + 2] * p.o[3 * j + 2];
    H[0] -= fac;

    // Eigenvector of m[k]: the largest column of (H - m_a)(H - m_b).
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double ma = m[(k + 1) % 3], mb = m[(k + 2) % 3];
        double A[9], B[9];
#pragma unroll
        for (int i = 0; i < 9; i++) {
            A[i] = H[i];
            B[i] = H[i];
        }
        A[0] -= ma; A[4] -= ma; A[8] -= ma;
        B[0] -= mb; B[4] -= mb; B[8] -= mb;
        double N[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                N[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
        int col = 0;
        double best = fabs(N[0]);
        if (fabs(N[4]) > best) { best = fabs(N[4]); col = 1; }
        if (fabs(N[8]) > best) { best = fabs(N[8]); col = 2; }
        double v0 = N[col], v1 = N[3 + col], v2 = N[6 + col];
        const double nrm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
        double inv = (nrm > 0.0) ? 1.0 / nrm : 0.0;
        // deterministic sign: largest component positive
        double big = v0;
        if (fabs(v1) > fabs(big)) big = v1;
        if (fabs(v2) > fabs(big)) big = v2;
        if (big < 0.0) inv = -inv;
        V[k] = v0 * inv;
        V[3 + k] = v1 * inv;
        V[6 + k] = v2 * inv;
    }
    // right-handed basis (det V = +1): every overlap T_l = V_{l+1}^T V_l is then a
    // rotation, which the propagation kernels rely on to rebuild a column
    const double det = V[0] * (V[4] * V[8] - V[5] * V[7]) - V[1] * (V[3] * V[8] - V[5] * V[6]) +
                       V[2] * (V[3] * V[7] - V[4] * V[6]);
    if (det < 0.0) {
        V[2] = -V[2];
        V[5] = -V[5];
        V[8] = -V[8];
    }
}

// Phase rate of eigenvalue k relative to eigenvalue 0, in turns per km:
// the reference's phase -LoEfac * m_k * L / E (physics.hpp:461-467) with the
// per-layer common phase of m_0 removed, divided by 2*pi.
CP3_HD double phase_turns_per_km(double mk, double m0, double E) {
    return -kLoEfac * (mk - m0) / E / kTwoPi;
}

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

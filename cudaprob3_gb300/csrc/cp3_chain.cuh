// Amplitude of one (cosine, energy) pair, written once for both arithmetic
// policies of cp3_arith.cuh.
//
// Reference behaviour (physics.hpp:645-677): the atmosphere segment A_0 is
// followed by shells 1..M-1 inbound, the innermost shell M (full chord), the
// same shells outbound, giving  S = A_1..A_{M-1} A_M A_{M-1}..A_1 A_0.  In the
// real eigen-basis every A_l = V_l D_l V_l^T is complex symmetric, so the
// outbound product is the transpose of the inbound one and
//
//   S_r = V_1 (Y^T D_M Y) T_0 D_0 V_0^T,   Y = T_{M-1} D_{M-1} ... T_1 D_1,
//
// with T_l = V_{l+1}^T V_l.  M = 0 (cos >= 0, atmosphere only, physics.hpp:562)
// gives S_r = V_0 D_0 V_0^T.  Finally S_f = W S_r W^dagger and
// P(in -> out) = |S_f[out][in]|^2 (physics.hpp:682-691).
#pragma once

#include "cp3_arith.cuh"

namespace cp3 {

// Src provides, for the current pair:
//   void phase(int l, R& c1, R& s1, R& n1, R& c2, R& s2, R& n2)  e^{i psi_k}, n = -s
//   R T(int l, int i, int j)    overlap V_{l+1}^T V_l
//   R V0(int i, int j), V1(int i, int j)
template <class P, class Src>
__device__ __forceinline__ void real_basis_amplitude(const Src& src, int M, typename P::C S[9]) {
    using R = typename P::R;
    using C = typename P::C;
    R c1, s1, n1, c2, s2, n2;
    if (M == 0) {
        src.phase(0, c1, s1, n1, c2, s2, n2);
        C X[9];  // X[3j+k] = V0(j,k) D_k
#pragma unroll
        for (int j = 0; j < 3; j++) {
            X[3 * j] = P::creal(src.V0(j, 0));
            X[3 * j + 1] = P::mulRC(src.V0(j, 1), C{c1, s1});
            X[3 * j + 2] = P::mulRC(src.V0(j, 2), C{c2, s2});
        }
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) {
                const C v = P::dotRC(src.V0(i, 0), src.V0(i, 1), src.V0(i, 2), X[3 * j], X[3 * j + 1],
                                     X[3 * j + 2]);
                S[3 * i + j] = v;
                S[3 * j + i] = v;
            }
        return;
    }
    C Y[9];
    if (M >= 2) {
        src.phase(1, c1, s1, n1, c2, s2, n2);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            Y[3 * i] = P::creal(src.T(1, i, 0));
            Y[3 * i + 1] = P::mulRC(src.T(1, i, 1), C{c1, s1});
            Y[3 * i + 2] = P::mulRC(src.T(1, i, 2), C{c2, s2});
        }
        for (int l = 2; l < M; l++) {
            src.phase(l, c1, s1, n1, c2, s2, n2);
            const R t00 = src.T(l, 0, 0), t01 = src.T(l, 0, 1), t02 = src.T(l, 0, 2);
            const R t10 = src.T(l, 1, 0), t11 = src.T(l, 1, 1), t12 = src.T(l, 1, 2);
            const R t20 = src.T(l, 2, 0), t21 = src.T(l, 2, 1), t22 = src.T(l, 2, 2);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const C z0 = Y[j];
                const C z1 = P::mulPhase(Y[3 + j], c1, s1, n1);
                const C z2 = P::mulPhase(Y[6 + j], c2, s2, n2);
                Y[j] = P::dotRC(t00, t01, t02, z0, z1, z2);
                Y[3 + j] = P::dotRC(t10, t11, t12, z0, z1, z2);
                Y[6 + j] = P::dotRC(t20, t21, t22, z0, z1, z2);
            }
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) Y[i] = P::cz();
        Y[0] = Y[4] = Y[8] = P::creal(P::one());
    }
    // G = Y^T D_M Y (symmetric)
    src.phase(M, c1, s1, n1, c2, s2, n2);
    C G[6];  // 00 01 02 11 12 22
    {
        C Z[9];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Z[j] = Y[j];
            Z[3 + j] = P::mulPhase(Y[3 + j], c1, s1, n1);
            Z[6 + j] = P::mulPhase(Y[6 + j], c2, s2, n2);
        }
        int g = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) G[g++] = P::dotCC(Y[i], Y[3 + i], Y[6 + i], Z[j], Z[3 + j], Z[6 + j]);
    }
    // K = G T_0 D_0
    src.phase(0, c1, s1, n1, c2, s2, n2);
    C K[9];
    {
        const C g00 = G[0], g01 = G[1], g02 = G[2], g11 = G[3], g12 = G[4], g22 = G[5];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const R a = src.T(0, 0, j), b = src.T(0, 1, j), c = src.T(0, 2, j);
            C k0 = P::dotRC(a, b, c, g00, g01, g02);
            C k1 = P::dotRC(a, b, c, g01, g11, g12);
            C k2 = P::dotRC(a, b, c, g02, g12, g22);
            if (j == 1) {
                k0 = P::mulPhase(k0, c1, s1, n1);
                k1 = P::mulPhase(k1, c1, s1, n1);
                k2 = P::mulPhase(k2, c1, s1, n1);
            } else if (j == 2) {
                k0 = P::mulPhase(k0, c2, s2, n2);
                k1 = P::mulPhase(k1, c2, s2, n2);
                k2 = P::mulPhase(k2, c2, s2, n2);
            }
            K[j] = k0;
            K[3 + j] = k1;
            K[6 + j] = k2;
        }
    }
    // S_r = V_1 K V_0^T
    C S1[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            S1[3 * i + j] = P::dotRC(src.V1(i, 0), src.V1(i, 1), src.V1(i, 2), K[j], K[3 + j], K[6 + j]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            S[3 * i + j] = P::dotRC(src.V0(j, 0), src.V0(j, 1), src.V0(j, 2), S1[3 * i], S1[3 * i + 1],
                                    S1[3 * i + 2]);
}

// S_f = W S_r W^dagger with W = R23 diag(1, 1, e^{i dcp}), in place.
template <class P>
__device__ __forceinline__ void to_flavour(typename P::C S[9], typename P::R c23, typename P::R s23,
                                           typename P::R cd, typename P::R sd) {
    // diag(1,1,e^{i d}) S diag(1,1,e^{-i d})
    S[6] = P::mulPhase(S[6], cd, sd, -sd);
    S[7] = P::mulPhase(S[7], cd, sd, -sd);
    S[2] = P::mulPhase(S[2], cd, -sd, sd);
    S[5] = P::mulPhase(S[5], cd, -sd, sd);
    // R23 from the left (rows 1, 2), then R23^T from the right (columns 1, 2)
#pragma unroll
    for (int j = 0; j < 3; j++) P::rot(c23, s23, S[3 + j], S[6 + j]);
#pragma unroll
    for (int i = 0; i < 3; i++) P::rot(c23, s23, S[3 * i + 1], S[3 * i + 2]);
}

}  // namespace cp3

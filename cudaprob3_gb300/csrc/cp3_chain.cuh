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
// gives S_r = V_0 D_0 V_0^T.  The flavour amplitude is S_f = W S_r W^dagger and
// P(in -> out) = |S_f[out][in]|^2 (physics.hpp:682-691); W enters only through
// the per-energy tables Lambda' = rows e, mu of W V_1 and
// Gamma' = columns e, mu of V_0^T W^dagger.
#pragma once

#include "cp3_arith.cuh"

namespace cp3 {

// Y = T_{M-1} D_{M-1} ... T_1 D_1 (row-major, Y[3 i + j]) of a pair that
// crosses M >= 1 shells.
template <class P, class Src>
__device__ __forceinline__ void chain_Y(const P& ar, const Src& src, int M, typename P::C Y[9]) {
    using R = typename P::R;
    using C = typename P::C;
    R c1, s1, n1, c2, s2, n2;
    if (M >= 2) {
        // Only columns 0 and 1 of Y are propagated; Y is unitary with
        // det Y = prod_l det(T_l) det(D_l) = e^{2 pi i sum_l (t1 + t2)_l}
        // (right-handed eigen-bases make det T_l = 1), so column 2 is
        // det(Y) conj(col0 x col1).
        typename Src::Turns phi;
        src.phase_acc(1, c1, s1, n1, c2, s2, n2, phi);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            Y[3 * i] = P::creal(src.T(1, i, 0));
            Y[3 * i + 1] = ar.mulRC(src.T(1, i, 1), C{c1, s1});
        }
        // unrolled by four: the compiler then overlaps one layer's phases
        // with another's products and needs no register moves between
        // iterations (measured on the 4096^2 grid, same bits: by two, 40
        // fewer IMAD per pair and 1.7 % faster than no unrolling; by four,
        // with the grouped table layout, no spill and 0.8 % faster again)
#pragma unroll 4
        for (int l = 2; l < M; l++) {
            src.phase_acc(l, c1, s1, n1, c2, s2, n2, phi);
            const R t00 = src.T(l, 0, 0), t01 = src.T(l, 0, 1), t02 = src.T(l, 0, 2);
            const R t10 = src.T(l, 1, 0), t11 = src.T(l, 1, 1), t12 = src.T(l, 1, 2);
            const R t20 = src.T(l, 2, 0), t21 = src.T(l, 2, 1), t22 = src.T(l, 2, 2);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const C z0 = Y[j];
                const C z1 = ar.mulPhase(Y[3 + j], c1, s1, n1);
                const C z2 = ar.mulPhase(Y[6 + j], c2, s2, n2);
                Y[j] = ar.dotRC(t00, t01, t02, z0, z1, z2);
                Y[3 + j] = ar.dotRC(t10, t11, t12, z0, z1, z2);
                Y[6 + j] = ar.dotRC(t20, t21, t22, z0, z1, z2);
            }
        }
        R dc, ds;
        src.turns_phase(phi, dc, ds);
        if (src.det_flip(M)) {  // columns 0 and 1 carry the sign of the negated overlaps
            dc = -dc;
            ds = -ds;
        }
        Y[2] = ar.mulPhase(ar.crossConj(Y[3], Y[6], Y[4], Y[7]), dc, ds, -ds);
        Y[5] = ar.mulPhase(ar.crossConj(Y[6], Y[0], Y[7], Y[1]), dc, ds, -ds);
        Y[8] = ar.mulPhase(ar.crossConj(Y[0], Y[3], Y[1], Y[4]), dc, ds, -ds);
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) Y[i] = P::cz();
        Y[0] = Y[4] = Y[8] = P::creal(P::one());
    }
}

// G = Y^T D_M Y (symmetric, entries 00 01 02 11 12 22) for the chain Y of
// a pair that crosses M >= 1 shells.
template <class P, class Src>
__device__ __forceinline__ void gram_G(const P& ar, const Src& src, int M, const typename P::C Y[9],
                                       typename P::C G[6]) {
    using R = typename P::R;
    using C = typename P::C;
    R c1, s1, n1, c2, s2, n2;
    src.phase(M, c1, s1, n1, c2, s2, n2);
    {
        C Z[9];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Z[j] = Y[j];
            Z[3 + j] = ar.mulPhase(Y[3 + j], c1, s1, n1);
            Z[6 + j] = ar.mulPhase(Y[6 + j], c2, s2, n2);
        }
        int g = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++) G[g++] = ar.dotCC(Y[i], Y[3 + i], Y[6 + i], Z[j], Z[3 + j], Z[6 + j]);
    }
}

template <class P, class Src>
__device__ __forceinline__ void chain_G(const P& ar, const Src& src, int M, typename P::C G[6]) {
    typename P::C Y[9];
    chain_Y(ar, src, M, Y);
    gram_G(ar, src, M, Y, G);
}

// Src provides, for the current pair:
//   void phase(int l, R& c1, R& s1, R& n1, R& c2, R& s2, R& n2)  e^{i psi_k}, n = -s
//   void phase_acc(..., Turns& acc)   the same, adding psi_1 + psi_2 (turns) to acc
//   void turns_phase(const Turns& acc, R& c, R& s)               e^{2 pi i acc}
//   void phase_len(int l, Len L, R& c1, ...)   e^{i psi_k} of layer l for a given length
//   R T(int l, int i, int j)     overlap V_{l+1}^T V_l (the mixed tables: negated for odd l)
//   bool det_flip(int M)         whether the chain over layers 1 .. M-1 negated Y
//   R La(int j)                  row 0 of W V_1 (real)
//   C Lb(int j)                  row 1 of W V_1
//   R Ga(int k)                  column 0 of V_0^T W^dagger (real)
//   C Gb(int k)                  column 1 of V_0^T W^dagger
//
// Only the 2x2 block S_f[out][in], out, in in {e, mu}, is formed: S_f is
// unitary, so the 3x3 matrix of |S_f|^2 is doubly stochastic and its other
// five entries follow from this block (complete_probabilities).
template <class P, class Src>
__device__ __forceinline__ void flavour_block(const P& ar, const Src& src, int M, typename P::C B[4]) {
    using R = typename P::R;
    using C = typename P::C;
    // The chain first: nothing of the atmosphere segment is live during the
    // layer loop (fewer registers across it).  The block is
    // Lambda' G X' with G = Y^T D_M Y and X' = T_0 D_0 Gamma' (3x2), formed in
    // one of two orders (same products up to rounding):
    //   G, then X = G X', then Lambda' X: 156 products after the chain; Y is
    //     dead before X' is formed (the Q1.30 path: no spill at 64 registers);
    //   by rows r_k of Y: a_k = Lambda' r_k, b_k = X'^T r_k and
    //     block = sum_k d_k a_k b_k^T, each entry rounded once: 147 products,
    //     but Y stays live beside X' (the FP64 path, which has the registers:
    //     2 % faster there; 24 bytes of spill and no gain on the Q1.30 path).
    constexpr bool by_rows = P::kBlockByRows;
    C Y[9];
    C G[6];  // 00 01 02 11 12 22 (first order only)
    if (M > 0) {
        chain_Y(ar, src, M, Y);
        if constexpr (!by_rows) gram_G(ar, src, M, Y, G);
    }
    R c1, s1, n1, c2, s2, n2;
    src.phase(0, c1, s1, n1, c2, s2, n2);
    C g0[3], g1[3];  // D_0 Gamma': columns 0 and 1
    g0[0] = P::creal(src.Ga(0));
    g0[1] = ar.mulRC(src.Ga(1), C{c1, s1});
    g0[2] = ar.mulRC(src.Ga(2), C{c2, s2});
    g1[0] = src.Gb(0);
    g1[1] = ar.mulPhase(src.Gb(1), c1, s1, n1);
    g1[2] = ar.mulPhase(src.Gb(2), c2, s2, n2);
    if (M == 0) {
        // S_r = V_0 D_0 V_0^T, so the block is Gamma'^dagger (D_0 Gamma')
        const C a0 = P::creal(src.Ga(0)), a1 = P::creal(src.Ga(1)), a2 = P::creal(src.Ga(2));
        const C b0 = P::conj(src.Gb(0)), b1 = P::conj(src.Gb(1)), b2 = P::conj(src.Gb(2));
        B[0] = ar.dotCC(a0, a1, a2, g0[0], g0[1], g0[2]);
        B[1] = ar.dotCC(a0, a1, a2, g1[0], g1[1], g1[2]);
        B[2] = ar.dotCC(b0, b1, b2, g0[0], g0[1], g0[2]);
        B[3] = ar.dotCC(b0, b1, b2, g1[0], g1[1], g1[2]);
        return;
    }
    C x0[3], x1[3];  // X' = T_0 (D_0 Gamma')
#pragma unroll
    for (int i = 0; i < 3; i++) {
        x0[i] = ar.dotRC(src.T(0, i, 0), src.T(0, i, 1), src.T(0, i, 2), g0[0], g0[1], g0[2]);
        x1[i] = ar.dotRC(src.T(0, i, 0), src.T(0, i, 1), src.T(0, i, 2), g1[0], g1[1], g1[2]);
    }
    if constexpr (by_rows) {
        // every factor is a dot product of unit vectors (|.| <= 1, as the
        // Gauss products need); row 0 of W V_1 is real, row 1 complex
        C a0[3], a1[3], b0[3], b1[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            b0[k] = ar.dotCC(Y[3 * k], Y[3 * k + 1], Y[3 * k + 2], x0[0], x0[1], x0[2]);
            b1[k] = ar.dotCC(Y[3 * k], Y[3 * k + 1], Y[3 * k + 2], x1[0], x1[1], x1[2]);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            a0[k] = ar.dotRC(src.La(0), src.La(1), src.La(2), Y[3 * k], Y[3 * k + 1], Y[3 * k + 2]);
            a1[k] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), Y[3 * k], Y[3 * k + 1], Y[3 * k + 2]);
        }
        src.phase(M, c1, s1, n1, c2, s2, n2);
        a0[1] = ar.mulPhase(a0[1], c1, s1, n1);
        a1[1] = ar.mulPhase(a1[1], c1, s1, n1);
        a0[2] = ar.mulPhase(a0[2], c2, s2, n2);
        a1[2] = ar.mulPhase(a1[2], c2, s2, n2);
        B[0] = ar.dotCC(a0[0], a0[1], a0[2], b0[0], b0[1], b0[2]);
        B[1] = ar.dotCC(a0[0], a0[1], a0[2], b1[0], b1[1], b1[2]);
        B[2] = ar.dotCC(a1[0], a1[1], a1[2], b0[0], b0[1], b0[2]);
        B[3] = ar.dotCC(a1[0], a1[1], a1[2], b1[0], b1[1], b1[2]);
    } else {
        // X = G X' (3x2), then the block = Lambda' X
        C X0[3], X1[3];
        X0[0] = ar.dotCC(G[0], G[1], G[2], x0[0], x0[1], x0[2]);
        X0[1] = ar.dotCC(G[1], G[3], G[4], x0[0], x0[1], x0[2]);
        X0[2] = ar.dotCC(G[2], G[4], G[5], x0[0], x0[1], x0[2]);
        X1[0] = ar.dotCC(G[0], G[1], G[2], x1[0], x1[1], x1[2]);
        X1[1] = ar.dotCC(G[1], G[3], G[4], x1[0], x1[1], x1[2]);
        X1[2] = ar.dotCC(G[2], G[4], G[5], x1[0], x1[1], x1[2]);
        B[0] = ar.dotRC(src.La(0), src.La(1), src.La(2), X0[0], X0[1], X0[2]);
        B[1] = ar.dotRC(src.La(0), src.La(1), src.La(2), X1[0], X1[1], X1[2]);
        B[2] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), X0[0], X0[1], X0[2]);
        B[3] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), X1[0], X1[1], X1[2]);
    }
}

// Probabilities of one pair averaged over production heights h with weights
// w_h (sum 1).  Only the atmosphere segment depends on h (physics.hpp:613-616),
// so the block factors as B(h) = R D_0(h) Gamma' with R = Lambda' G T_0 (or
// Gamma'^dagger when no shell is crossed): the chain runs once, each height
// costs one phase pair and four phase sums.  `lenh` holds the pair's
// atmosphere length at every height in the Src's length format; the averaged
// |B|^2 are completed to the nine probabilities (the completion is linear).
template <class P, class Src, class LenT, class WT>
__device__ __forceinline__ void flavour_probs_heights(const P& ar, const Src& src, int M, int H, const LenT* lenh,
                                                      const WT* w, typename P::Acc out[9]) {
    using R = typename P::R;
    using C = typename P::C;
    using A = typename P::Acc;
    C R0[3], R1[3];
    if (M == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            R0[k] = P::creal(src.Ga(k));
            R1[k] = P::conj(src.Gb(k));
        }
    } else {
        C G[6];
        chain_G(ar, src, M, G);
        // rows of Lambda' G (G symmetric: column j = row j)
        C l0[3], l1[3];
        l0[0] = ar.dotRC(src.La(0), src.La(1), src.La(2), G[0], G[1], G[2]);
        l0[1] = ar.dotRC(src.La(0), src.La(1), src.La(2), G[1], G[3], G[4]);
        l0[2] = ar.dotRC(src.La(0), src.La(1), src.La(2), G[2], G[4], G[5]);
        l1[0] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), G[0], G[1], G[2]);
        l1[1] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), G[1], G[3], G[4]);
        l1[2] = ar.dotCC(src.Lb(0), src.Lb(1), src.Lb(2), G[2], G[4], G[5]);
        // times T_0: R[r][k] = sum_j (Lambda' G)[r][j] T_0[j][k]
#pragma unroll
        for (int k = 0; k < 3; k++) {
            R0[k] = ar.dotRC(src.T(0, 0, k), src.T(0, 1, k), src.T(0, 2, k), l0[0], l0[1], l0[2]);
            R1[k] = ar.dotRC(src.T(0, 0, k), src.T(0, 1, k), src.T(0, 2, k), l1[0], l1[1], l1[2]);
        }
    }
    // B(h)[r][c] = sum_k R_r[k] d_k(h) Gamma'_c[k] = sum_k Q_rc[k] d_k(h) with
    // d_0 = 1: the products Q_rc[k] = R_r[k] Gamma'_c[k] do not depend on the
    // height (30 products once per pair), so a height costs two phases and
    // four phase sums (24 products) instead of forming D_0(h) Gamma' and
    // four 3-term dot products (46)
    C Q00[3], Q01[3], Q10[3], Q11[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Q00[k] = ar.mulRC(src.Ga(k), R0[k]);
        Q01[k] = ar.mulCC(R0[k], src.Gb(k));
        Q10[k] = ar.mulRC(src.Ga(k), R1[k]);
        Q11[k] = ar.mulCC(R1[k], src.Gb(k));
    }
    A q00 = 0, q01 = 0, q10 = 0, q11 = 0;
    for (int h = 0; h < H; h++) {
        R c1, s1, n1, c2, s2, n2;
        src.phase_len(0, lenh[h], c1, s1, n1, c2, s2, n2);
        const A wh = (A)w[h];
        q00 += wh * P::prob(ar.phaseSum(Q00[0], Q00[1], Q00[2], c1, s1, c2, s2));
        q01 += wh * P::prob(ar.phaseSum(Q01[0], Q01[1], Q01[2], c1, s1, c2, s2));
        q10 += wh * P::prob(ar.phaseSum(Q10[0], Q10[1], Q10[2], c1, s1, c2, s2));
        q11 += wh * P::prob(ar.phaseSum(Q11[0], Q11[1], Q11[2], c1, s1, c2, s2));
    }
    P::complete_avg(q00, q01, q10, q11, out);
}

}  // namespace cp3

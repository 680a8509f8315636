// Per-tile and per-thread device code shared by the single-grid kernels
// (cp3_kernels.cu) and the batched persistent kernel (cp3_batch.cu).
//
//   prep_energy_layer  eigen-solve of one (energy, layer) (double-float for
//                      the mixed tables, FP64 for the FP64 ones) and the
//                      mixed/FP64 table entries derived from it
//   prep_overlap(_v)   T_l = V_{l+1}^T V_l of one (energy, layer)
//   prep_cosine_layer  segment length of one (trajectory, layer)
//   process_tile       one block's tile: TE energies x a chunk of cosines of
//                      one grid -> 9 probability planes
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "cp3_chain.cuh"
#include "cp3_check.cuh"
#include "cp3_internal.h"
#include "cp3_physics.cuh"

namespace cp3 {

// Tables of one grid as the prep kernels write them (see cp3_kernels.cu).
struct GridTables {
    void* tab;  // tile-major [n_en_pad/TE][nl][W][TE]
    void* pe;   // [18][n_en_pad]
    void* len;  // [n_cos][nl_pad]
    int n_en_pad, te, nl, nl_pad;
};

// Layout of the mixed tables' words, so that a lane reads its words with 16-byte
// loads.  An (energy-tile, layer) block of the mixed table holds 13 words per
// energy of the tile (te energies): words 0-11 as three groups of four
// consecutive words per energy ([3][te][4]), word 12 on its own ([te]).  The
// per-energy table in shared memory (18 words) is four groups of four
// ([4][te][4]) and a pair ([te][2]).  Both take exactly the space of the
// word-major layout ([13][te], [18][te]).
__host__ __device__ inline int mixed_word_offset(int w, int lane, int te) {
    return w < 12 ? (w >> 2) * 4 * te + lane * 4 + (w & 3) : 12 * te + lane;
}
__host__ __device__ inline int mixed_pe_offset(int w, int lane, int te) {
    return w < 16 ? (w >> 2) * 4 * te + lane * 4 + (w & 3) : 16 * te + lane * 2 + (w - 16);
}

// Thread (l, e) of the energy part: eigen-solve of layer l at energy E, writes
// kappa (and Lambda'/Gamma' for l = 0, 1), leaves the eigenvectors in `vme`
// (shared memory) for the overlap pass and, if `m_out` is given, the
// eigenvalues there.  The mixed tables (Q1.30 words, float hi/lo pairs) come
// from the double-float solve on the FP32 pipes (layer_eigen_df), and `vme`
// then holds the eigenvectors as double-float pairs in the same 8-byte
// slots; the FP64 tables from the FP64 solve.
template <bool MIXED>
__device__ __forceinline__ void prep_energy_layer(const OscParams& osc, double E, double rhoye, int l, int e,
                                                  const GridTables& g, double* vme, double* m_out = nullptr) {
    const int te = g.te, tile = e / te, lane = e % te;
    const int W = MIXED ? kMixedWords : kFp64Words;
    if (!(check_ok(kSitePrepTab, tile, g.n_en_pad / te) && check_ok(kSitePrepLayer, l, g.nl))) return;
    const size_t block = ((size_t)tile * g.nl + l) * W * te;  // this (tile, layer)'s words
    const size_t base = block + lane;
    if constexpr (MIXED) {
        const DF Ed = df_from_double(E);
        DF m[3], V[9];
        layer_eigen_df(osc, Ed, df_from_double(rhoye), m, V);
#pragma unroll
        for (int w = 0; w < 9; w++) df_store(vme + w, V[w]);
        if (m_out)
#pragma unroll
            for (int k = 0; k < 3; k++) m_out[k] = df_to_double(m[k]);
        const DF fE = df_rate_factor(Ed);
        const DF k1 = df_mul(df_sub(m[1], m[0]), fE);
        const DF k2 = df_mul(df_sub(m[2], m[0]), fE);
        int* t = (int*)g.tab + block;
        t[mixed_word_offset(9, lane, te)] = __float_as_int(k1.hi);
        t[mixed_word_offset(10, lane, te)] = __float_as_int(k1.lo);
        t[mixed_word_offset(11, lane, te)] = __float_as_int(k2.hi);
        t[mixed_word_offset(12, lane, te)] = __float_as_int(k2.lo);
        if (l <= 1) {
            // per energy: Gamma' = columns e, mu of V_0^T W^dagger (l = 0) and
            // Lambda' = rows e, mu of W V_1 (l = 1), W = R23 diag(1, 1, e^{i dcp})
            const DF c23 = df_load(osc.c23_f), s23 = df_load(osc.s23_f);
            const DF s23cd = df_mul(s23, df_load(osc.cd_f));
            DF s23sd = df_mul(s23, df_load(osc.sd_f));
            if (l == 0) s23sd = df_neg(s23sd);  // e^{-i dcp} for Gamma', e^{+i dcp} for Lambda'
            int w[9];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                w[k] = q30_df(V[k]);
                w[3 + 2 * k] = q30_df(df_add(df_mul(c23, V[3 + k]), df_mul(s23cd, V[6 + k])));
                w[4 + 2 * k] = q30_df(df_mul(s23sd, V[6 + k]));
            }
            const int off = (l == 0) ? 9 : 0;
#pragma unroll
            for (int q = 0; q < 9; q++) ((int*)g.pe)[(size_t)(off + q) * g.n_en_pad + e] = w[q];
        }
    } else {
        double m[3], V[9];
        layer_eigen(osc, E, rhoye, m, V);
        for (int w = 0; w < 9; w++) vme[w] = V[w];
        if (m_out)
            for (int k = 0; k < 3; k++) m_out[k] = m[k];
        const double fE = phase_rate_factor(E);
        double* t = (double*)g.tab;
        t[base + 9 * (size_t)te] = (m[1] - m[0]) * fE;
        t[base + 10 * (size_t)te] = (m[2] - m[0]) * fE;
        if (l <= 1) {
            const double sg = (l == 0) ? -1.0 : 1.0;
            double w[9];
            for (int k = 0; k < 3; k++) {
                w[k] = V[k];
                w[3 + 2 * k] = osc.c23 * V[3 + k] + osc.s23 * osc.cd * V[6 + k];
                w[4 + 2 * k] = sg * osc.s23 * osc.sd * V[6 + k];
            }
            const int off = (l == 0) ? 9 : 0;
            for (int q = 0; q < 9; q++) ((double*)g.pe)[(size_t)(off + q) * g.n_en_pad + e] = w[q];
        }
    }
}

// Overlap pass of thread (l, e): T_l = V_{l+1}^T V_l from its own eigenvectors
// v and the next layer's vn (double-float pairs for the mixed tables); the
// innermost layer has no successor and keeps the identity.  The mixed tables
// hold -T_l for odd l: the Q1.30 chain rounds down (floor), and with the sign
// of Y alternating from layer to layer the rounding errors of consecutive
// layers point in opposite directions in the true frame instead of adding up
// (MixedSrc::det_flip restores the sign of the third column).
template <bool MIXED>
__device__ __forceinline__ void prep_overlap_v(int l, int e, const GridTables& g, const double* v, const double* vn) {
    const int te = g.te, tile = e / te, lane = e % te;
    const int W = MIXED ? kMixedWords : kFp64Words;
    if (!(check_ok(kSitePrepTab, tile, g.n_en_pad / te) && check_ok(kSitePrepLayer, l, g.nl))) return;
    const size_t block = ((size_t)tile * g.nl + l) * W * te;
    const size_t base = block + lane;
    const bool last = !(l + 1 < g.nl);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if constexpr (MIXED) {
                const DF tij = last ? DF{(i == j) ? 1.0f : 0.0f, 0.0f}
                                    : df_add(df_add(df_mul(df_read(vn + i), df_read(v + j)),
                                                    df_mul(df_read(vn + 3 + i), df_read(v + 3 + j))),
                                             df_mul(df_read(vn + 6 + i), df_read(v + 6 + j)));
                const int q = q30_df(tij);
                ((int*)g.tab)[block + mixed_word_offset(3 * i + j, lane, te)] = (l & 1) ? -q : q;
            } else {
                const double tij = last ? (i == j ? 1.0 : 0.0) : vn[i] * v[j] + vn[3 + i] * v[3 + j] + vn[6 + i] * v[6 + j];
                ((double*)g.tab)[base + (size_t)(3 * i + j) * te] = tij;
            }
        }
}

// The same with the layers' eigenvectors in shared memory ([layer][9], the
// next layer's right after this one's).
template <bool MIXED>
__device__ __forceinline__ void prep_overlap(int l, int e, const GridTables& g, const double* vme) {
    prep_overlap_v<MIXED>(l, e, g, vme, vme + 9);
}

// Segment length of layer l of trajectory c (zero beyond M).  One thread per
// (cosine, layer): a thread running all layers in sequence would be a chain
// of some 25 FP64 square roots, far longer than any eigen-solve.
template <bool MIXED>
__device__ __forceinline__ void prep_cosine_layer(double cz, int M, const double* radii, double height_cm, int c,
                                                  int l, const GridTables& g) {
    // the chord of layer l reads the density rows up to M
    if (!(check_ok(kSitePrepLayer, M, g.nl) && check_ok(kSitePrepLen, l, g.nl_pad))) return;
    const double L = (l <= M) ? layer_length_km(radii, l, M, cz, path_length_cm(cz, height_cm)) : 0.0;
    const size_t idx = (size_t)c * g.nl_pad + l;
    if (MIXED) {
        const float h = f32_rn(L);
        ((float2*)g.len)[idx] = make_float2(h, f32_rn(L - f64_of(h)));
    } else {
        ((double*)g.len)[idx] = L;
    }
}

// ------------------------------------------------------------ propagate ----
template <int TE>
struct MixedSrc {
    const int* tab;    // shared: the tile's [nl][13 words][TE] in the grouped layout (mixed_word_offset)
    const int* pe;     // shared: [18 words][TE] in the grouped layout (mixed_pe_offset)
    const float2* len; // shared: this cosine's [nl_pad]
    const int4* ptab;  // shared: 257 (Q1.30 cos, sin, float cos, sin)
    int lane;          // the thread's energy within the tile
    static __device__ __forceinline__ int pick(int4 v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }
    // word w of layer l: words 0-11 come from 16-byte loads (the compiler
    // merges the loads of one group), word 12 from a 4-byte load
    __device__ __forceinline__ int word(int l, int w) const {
        if (w < 12) return pick(((const int4*)(tab + l * kMixedWords * TE))[(w >> 2) * TE + lane], w & 3);
        return tab[l * kMixedWords * TE + 12 * TE + lane];
    }
    __device__ __forceinline__ int pe_word(int w) const {
        if (w < 16) return pick(((const int4*)pe)[(w >> 2) * TE + lane], w & 3);
        const int2 v = ((const int2*)(pe + 16 * TE))[lane];
        return w == 16 ? v.x : v.y;
    }
    __device__ __forceinline__ int T(int l, int i, int j) const { return word(l, 3 * i + j); }
    // the chain over layers 1 .. M-1 crossed floor(M/2) negated overlaps
    __device__ __forceinline__ bool det_flip(int M) const { return (M >> 1) & 1; }
    __device__ __forceinline__ int La(int j) const { return pe_word(j); }
    __device__ __forceinline__ Q30::C Lb(int j) const { return Q30::C{pe_word(3 + 2 * j), pe_word(4 + 2 * j)}; }
    __device__ __forceinline__ int Ga(int k) const { return pe_word(9 + k); }
    __device__ __forceinline__ Q30::C Gb(int k) const { return Q30::C{pe_word(12 + 2 * k), pe_word(13 + 2 * k)}; }
    __device__ __forceinline__ void phase(int l, int& c1, int& s1, int& n1, int& c2, int& s2, int& n2) const {
        phase_len(l, len[l], c1, s1, n1, c2, s2, n2);
    }
    __device__ __forceinline__ void phase_len(int l, float2 L, int& c1, int& s1, int& n1, int& c2, int& s2,
                                              int& n2) const {
        phase_q30(__int_as_float(word(l, 9)), __int_as_float(word(l, 10)), L.x, L.y, ptab, c1, s1);
        phase_q30(__int_as_float(word(l, 11)), __int_as_float(word(l, 12)), L.x, L.y, ptab, c2, s2);
        n1 = -s1;
        n2 = -s2;
    }
    using Turns = TurnSum;
    __device__ __forceinline__ void phase_acc(int l, int& c1, int& s1, int& n1, int& c2, int& s2, int& n2,
                                              Turns& acc) const {
        const float2 L = len[l];
        float p1, e1, p2, e2;
        turns_product(__int_as_float(word(l, 9)), __int_as_float(word(l, 10)), L.x, L.y, p1, e1);
        turns_product(__int_as_float(word(l, 11)), __int_as_float(word(l, 12)), L.x, L.y, p2, e2);
        const float u1 = p1 - rintf(p1), u2 = p2 - rintf(p2);
        int j1, j2;
        float d1, d2;
        turns_q30_u(u1, e1, ptab, c1, s1, j1, d1);
        turns_q30_u(u2, e2, ptab, c2, s2, j2, d2);
        acc.add(j1, d1);
        acc.add(j2, d2);
        n1 = -s1;
        n2 = -s2;
    }
    __device__ __forceinline__ void turns_phase(const Turns& acc, int& c, int& s) const {
        float u, e;
        acc.split(u, e);
        turns_q30_u(u, e, ptab, c, s);
    }
};

template <int TE>
struct F64Src {
    const double* tab;  // shared: [nl][11][TE], offset by lane
    const double* pe;
    const double* len;
    const double2* ptab;  // shared: 257 (cos, sin) of 2*pi*j/256
    __device__ __forceinline__ double T(int l, int i, int j) const { return tab[(l * kFp64Words + 3 * i + j) * TE]; }
    __device__ __forceinline__ bool det_flip(int) const { return false; }
    __device__ __forceinline__ double La(int j) const { return pe[j * TE]; }
    __device__ __forceinline__ F64::C Lb(int j) const { return F64::C{pe[(3 + 2 * j) * TE], pe[(4 + 2 * j) * TE]}; }
    __device__ __forceinline__ double Ga(int k) const { return pe[(9 + k) * TE]; }
    __device__ __forceinline__ F64::C Gb(int k) const { return F64::C{pe[(12 + 2 * k) * TE], pe[(13 + 2 * k) * TE]}; }
    __device__ __forceinline__ void phase(int l, double& c1, double& s1, double& n1, double& c2, double& s2,
                                          double& n2) const {
        phase_len(l, len[l], c1, s1, n1, c2, s2, n2);
    }
    __device__ __forceinline__ void phase_len(int l, double L, double& c1, double& s1, double& n1, double& c2,
                                              double& s2, double& n2) const {
        const double* k = tab + (l * kFp64Words + 9) * TE;
        phase_f64(k[0], L, ptab, c1, s1);
        phase_f64(k[TE], L, ptab, c2, s2);
        n1 = -s1;
        n2 = -s2;
    }
    // Sum of phases in turns as (sum of the table indices j) / 256 + (sum of
    // the exact remainders d): the integer part is exact, the remainders stay
    // below 1/512 each.
    struct Turns {
        unsigned j = 0;  // mod 2^32: only j mod 256 is read
        double d = 0.0;
    };
    __device__ __forceinline__ void phase_acc(int l, double& c1, double& s1, double& n1, double& c2, double& s2,
                                              double& n2, Turns& acc) const {
        const double L = len[l];
        const double* k = tab + (l * kFp64Words + 9) * TE;
        int j1, j2;
        double d1, d2;
        reduce_product_f64(k[0], L, j1, d1);
        reduce_product_f64(k[TE], L, j2, d2);
        sincos_reduced_f64(j1, d1, ptab, c1, s1);
        sincos_reduced_f64(j2, d2, ptab, c2, s2);
        n1 = -s1;
        n2 = -s2;
        acc.j += (unsigned)j1 + (unsigned)j2;
        acc.d += d1 + d2;
    }
    __device__ __forceinline__ void turns_phase(const Turns& acc, double& c, double& s) const {
        sincos_turns_f64(fma((double)(int)(acc.j & 255u), 0.00390625, acc.d), ptab, c, s);
    }
};

// Copy `n16` 16-byte units from global to shared with the whole block.
__device__ __forceinline__ void block_copy16(void* dst, const void* src, int n16) {
    const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
    int4* d = (int4*)dst;
    const int4* s = (const int4*)src;
    for (int i = t; i < n16; i += nt) d[i] = __ldg(s + i);
}


// Shared-memory layout of one tile (bytes); `cchunk` bounds the cosine chunk.
struct TileSmem {
    size_t tab, pe, ptab, len, maxl, cbin, total;
};
__host__ __device__ inline TileSmem tile_smem(bool mixed, int te, int nl, int nl_pad, int cchunk) {
    const size_t word = mixed ? 4 : 8;
    const size_t W = mixed ? kMixedWords : kFp64Words;
    TileSmem t;
    t.tab = 0;
    t.pe = t.tab + (size_t)nl * W * te * word;
    t.ptab = t.pe + (size_t)kPerEWords * te * word;
    t.len = t.ptab + kPhaseTabBytes;  // mixed: int4 entries; FP64: double2 entries
    t.maxl = t.len + (size_t)cchunk * nl_pad * 8;
    t.cbin = t.maxl + (size_t)cchunk * 4;
    t.total = (t.cbin + (size_t)cchunk * 4 + 15) / 16 * 16;
    return t;
}

// One tile of one grid: energies [etile*TE, etile*TE + TE) and cosines
// [c0, c0 + ncl).  The block stages the tile's tables in shared memory and
// each (lane, group) thread walks its cosines.  The phase table must already
// be in shared memory (stage_phase_table).  Callers synchronise the block
// between consecutive tiles.
struct TileJob {
    const void* tab;   // grid's tile-major table
    const void* pe;    // grid's [18][n_en_pad]
    const void* len;   // grid's [n_cos][nl_pad]
    const int* maxl;   // grid's layer counts
    void* out;         // grid's [9][n_cos][n_en]
    int n_cos, n_en, n_en_pad;
    int etile, c0, ncl;
    // fused event rates (process_tile<..., RATES = true>): instead of the
    // planes, rate_b(c, E) = sum_a flux[a][c][E] P(a -> b) is summed into
    // hist[b][cbin[c]][ebin[E]] (bin -1: not histogrammed)
    const float* flux;  // [3][n_cos][n_en], planes whose bit is clear in flux_mask are not read
    int flux_mask;
    const int* cbin;    // [n_cos]
    const int* ebin;    // [n_en]
    double* hist;       // [3][n_cb][n_eb]
    int n_cb, n_eb;
    // production-height average (process_tile<..., kModeHeights>): the
    // atmosphere length of every cosine at each of n_h heights and the weights
    const void* lenh;   // [n_cos][n_h] float2 hi/lo (mixed) or double
    const void* hw;     // [n_h] float (mixed) or double, sum 1
    int n_h;
};

// What process_tile does with each pair's probabilities.
constexpr int kModePlanes = 0;   // store the nine planes
constexpr int kModeRates = 1;    // fused event-rate histograms
constexpr int kModeHeights = 2;  // planes averaged over production heights
constexpr int kModeBlock = 3;    // only the planes of the 2x2 flavour block (e->e, e->mu, mu->e, mu->mu);
                                 // the host derives the other five (unitarity)

// Adds one run of rates (the lanes' sums since the warp's cosine bin `cb`
// changed) to the histogram.  `cb` is warp-uniform (a warp's lanes share the
// cosine); `eb` is the lane's energy bin.  When the lanes of equal energy bin
// form contiguous groups (monotone binning), each group is summed by a
// segmented butterfly and its first lane adds it: one atomic per bin and
// flavour; otherwise every lane adds its own sums.  Called by whole warps.
template <class Acc>
__device__ __forceinline__ void flush_rates(Acc& s0, Acc& s1, Acc& s2, int cb, int eb, const TileJob& j) {
    const unsigned full = 0xffffffffu;
    if (cb >= 0) {
        const int lane = threadIdx.x & 31;
        const unsigned grp = __match_any_sync(full, eb);
        const int lo = __ffs(grp) - 1, hi = 31 - __clz(grp);
        const unsigned span = (hi - lo == 31) ? full : (((1u << (hi - lo + 1)) - 1u) << lo);
        if (__all_sync(full, grp == span)) {
            const int end = hi + 1;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const Acc o0 = __shfl_down_sync(full, s0, off);
                const Acc o1 = __shfl_down_sync(full, s1, off);
                const Acc o2 = __shfl_down_sync(full, s2, off);
                if (lane + off < end) {
                    s0 += o0;
                    s1 += o1;
                    s2 += o2;
                }
            }
            if (lane != lo) eb = -1;
        }
        if (eb >= 0 && check_ok(kSiteTileHist, cb, j.n_cb) && check_ok(kSiteTileHist, eb, j.n_eb)) {
            const size_t pl = (size_t)j.n_cb * j.n_eb;
            double* h = j.hist + (size_t)cb * j.n_eb + eb;
            atomicAdd(h, (double)s0);
            atomicAdd(h + pl, (double)s1);
            atomicAdd(h + 2 * pl, (double)s2);
        }
    }
    s0 = s1 = s2 = Acc(0);
}

// Rate of final flavour b at (ci, e) from the nine probabilities.
template <class Acc, class P>
__device__ __forceinline__ void add_rates(const TileJob& j, int ci, int e, const P* pr, Acc& s0, Acc& s1, Acc& s2) {
    const size_t plane = (size_t)j.n_cos * j.n_en, at = (size_t)ci * j.n_en + e;
    const Acc f0 = (j.flux_mask & 1) ? (Acc)__ldcs(j.flux + at) : Acc(0);
    const Acc f1 = (j.flux_mask & 2) ? (Acc)__ldcs(j.flux + plane + at) : Acc(0);
    const Acc f2 = (j.flux_mask & 4) ? (Acc)__ldcs(j.flux + 2 * plane + at) : Acc(0);
    s0 += f0 * (Acc)pr[0] + f1 * (Acc)pr[3] + f2 * (Acc)pr[6];
    s1 += f0 * (Acc)pr[1] + f1 * (Acc)pr[4] + f2 * (Acc)pr[7];
    s2 += f0 * (Acc)pr[2] + f1 * (Acc)pr[5] + f2 * (Acc)pr[8];
}

template <bool MIXED>
__device__ __forceinline__ void stage_phase_table(unsigned char* smem, const TileSmem& L, const int4* ptab) {
    const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
    int4* s = (int4*)(smem + L.ptab);
    for (int i = t; i < kPhaseTabN + 1; i += nt) s[i] = ptab[i];
}

template <bool MIXED, int TE, int MODE = kModePlanes>
__device__ __forceinline__ void process_tile(const TileJob& j, int nl, int nl_pad, unsigned char* smem,
                                             const TileSmem& L) {
    constexpr bool RATES = MODE == kModeRates;
    using Word = typename std::conditional<MIXED, int, double>::type;
    constexpr int W = MIXED ? kMixedWords : kFp64Words;
    // checked build: the tile must lie in the grid's tables and its cosine
    // rows in the grid and in the staged chunk (the same for every thread of
    // the block, so a bad tile is skipped by the whole block)
    if (!(check_ok(kSiteTileTab, j.etile, j.n_en_pad / TE) &&
          (j.ncl <= 0 || (check_ok(kSiteTileChunk, j.ncl - 1, (long long)((L.cbin - L.maxl) / 4)) &&
                          check_ok(kSiteTileLen, j.c0, j.n_cos) &&
                          check_ok(kSiteTileLen, (long long)j.c0 + j.ncl - 1, j.n_cos)))))
        return;
    Word* s_tab = (Word*)(smem + L.tab);
    Word* s_pe = (Word*)(smem + L.pe);
    const int4* s_ptab = (const int4*)(smem + L.ptab);
    unsigned char* s_len_raw = smem + L.len;
    int* s_maxl = (int*)(smem + L.maxl);
    const size_t tab_words = (size_t)nl * W * TE;
    block_copy16(s_tab, (const Word*)j.tab + (size_t)j.etile * tab_words, (int)(tab_words * sizeof(Word) / 16));
    {
        const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
        const Word* pe = (const Word*)j.pe;
        for (int i = t; i < kPerEWords * TE; i += nt) {
            const int w = i / TE, lane = i % TE;
            s_pe[MIXED ? mixed_pe_offset(w, lane, TE) : i] = pe[(size_t)w * j.n_en_pad + (size_t)j.etile * TE + lane];
        }
        const int nlen16 = j.ncl * nl_pad / 2;  // 8-byte entries, nl_pad even
        block_copy16(s_len_raw, (const unsigned char*)j.len + (size_t)j.c0 * nl_pad * 8, nlen16);
        for (int i = t; i < j.ncl; i += nt) s_maxl[i] = j.maxl[j.c0 + i];
        if (RATES) {
            int* s_cbin = (int*)(smem + L.cbin);
            for (int i = t; i < j.ncl; i += nt) s_cbin[i] = j.cbin[j.c0 + i];
        }
    }
    __syncthreads();

    const int lane = threadIdx.x;
    const int e = j.etile * TE + lane;
    const bool store = e < j.n_en;
    const size_t plane = (size_t)j.n_cos * j.n_en;
    // fused rates: per-lane sums of the current cosine-bin run (FP32 for the
    // mixed kernel: a run is a few cosines; FP64 for the FP64 kernel)
    using Acc = typename std::conditional<MIXED, float, double>::type;
    Acc r0 = 0, r1 = 0, r2 = 0;
    int run_cb = -1;
    const int my_eb = (RATES && store) ? j.ebin[e] : -1;
    // a warp whose energies all lie past the grid (the last, partial tile of
    // a grid whose energy count is not a multiple of TE) has nothing to do
    // (no barrier follows in this function; callers synchronise after it)
    if (j.etile * TE + (lane & ~31) >= j.n_en) return;
    for (int cl = threadIdx.y; cl < j.ncl; cl += blockDim.y) {
        const int M = CP3_IX(kSiteTileLayers, s_maxl[cl], nl);
        const int ci = j.c0 + cl;
        if (MIXED) {
            MixedSrc<TE> src{(const int*)s_tab, (const int*)s_pe, (const float2*)s_len_raw + (size_t)cl * nl_pad,
                             s_ptab, lane};
            const Q30 ar{};
            float pr[9];
            if (MODE == kModeHeights) {
                flavour_probs_heights<Q30>(ar, src, M, j.n_h, (const float2*)j.lenh + (size_t)ci * j.n_h,
                                           (const float*)j.hw, pr);
            } else {
                Q30::C B[4];
                flavour_block<Q30>(ar, src, M, B);
                Q30::complete(B, pr);
            }
            if (RATES) {
                const int cb = ((const int*)(smem + L.cbin))[cl];
                if (cb != run_cb) {
                    flush_rates(r0, r1, r2, run_cb, my_eb, j);
                    run_cb = cb;
                }
                if (cb >= 0 && my_eb >= 0) add_rates(j, ci, e, pr, r0, r1, r2);
            } else if (store) {
                float* out = (float*)j.out + (size_t)ci * j.n_en + e;
                if (MODE == kModeBlock) {
                    __stcs(out, pr[0]);
                    __stcs(out + plane, pr[1]);
                    __stcs(out + 3 * plane, pr[3]);
                    __stcs(out + 4 * plane, pr[4]);
                } else {
#pragma unroll
                    for (int t = 0; t < 9; t++) __stcs(out + (size_t)t * plane, pr[t]);
                }
            }
        } else {
            F64Src<TE> src{(const double*)s_tab + lane, (const double*)s_pe + lane,
                           (const double*)s_len_raw + (size_t)cl * nl_pad, (const double2*)s_ptab};
            const F64 ar{};
            double pr[9];
            if (MODE == kModeHeights) {
                flavour_probs_heights<F64>(ar, src, M, j.n_h, (const double*)j.lenh + (size_t)ci * j.n_h,
                                           (const double*)j.hw, pr);
            } else {
                F64::C B[4];
                flavour_block<F64>(ar, src, M, B);
                F64::complete(B, pr);
            }
            if (RATES) {
                const int cb = ((const int*)(smem + L.cbin))[cl];
                if (cb != run_cb) {
                    flush_rates(r0, r1, r2, run_cb, my_eb, j);
                    run_cb = cb;
                }
                if (cb >= 0 && my_eb >= 0) add_rates(j, ci, e, pr, r0, r1, r2);
            } else if (store) {
                double* out = (double*)j.out + (size_t)ci * j.n_en + e;
                if (MODE == kModeBlock) {
                    __stcs(out, pr[0]);
                    __stcs(out + plane, pr[1]);
                    __stcs(out + 3 * plane, pr[3]);
                    __stcs(out + 4 * plane, pr[4]);
                } else {
#pragma unroll
                    for (int t = 0; t < 9; t++) __stcs(out + (size_t)t * plane, pr[t]);
                }
            }
        }
    }
    if (RATES) flush_rates(r0, r1, r2, run_cb, my_eb, j);
}

}  // namespace cp3

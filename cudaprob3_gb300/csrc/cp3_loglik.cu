// Binned Poisson log-likelihood of the propagated probabilities and its
// gradient by a hand-written adjoint (reverse mode).
//
// No reference counterpart: CUDAProb3++ computes probabilities only.  The
// forward model per bin b = (cosine c, energy E) is
//   lambda_b = norm * (flux_e(E) P(e -> mu) + flux_mu(E) P(mu -> mu)),
//   LL = sum_b n_b ln lambda_b - lambda_b   (constant terms dropped),
// with P from the same propagation as the probability kernels (real eigen-basis,
// transpose-symmetric layer chain, 2x2 flavour block; cp3_chain.cuh).  The
// gradient is taken with respect to theta12, theta13, theta23, dCP, dm12sq,
// dm23sq and the density of every row of the body (caller's row order).
//
// Launches of one evaluation (captured in a CUDA graph together with the
// parameter upload and the result download):
//   ll_prep_kernel    eigen tables of every (energy, layer) (FP64, or the
//                     double-float solve writing the float tables of the mixed
//                     pair kernel) and segment lengths
//   ll_pair_kernel    one warp = one energy x 32 cosines; forward chain, LL and
//                     seeds, then the backward pass that recomputes each layer
//                     matrix from the tables (no per-layer storage: the chain is
//                     un-multiplied with T^T and conj(D)); per-(energy, layer)
//                     adjoints are summed over the warp's cosines with shuffles
//   ll_layer_kernel   three threads (rows) per (energy, layer), packed densely
//                     over energies: sums the warps' partials and
//                     back-propagates through the layer's FP64
//                     eigen-decomposition to the parameters
// The per-energy rows land in mapped host memory; the host sums them over the
// energies in a fixed order (deterministic) after the graph completes.
// Precision: FP64 does every step in double; MIXED solves the layers in
// double-float arithmetic, runs ll_pair_kernel in FP32 (phases in
// double-float) on float tables, sums its float partials
// over the cosine chunks by compensated FP32 sums and does the eigen
// back-propagation in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "cudaprob3_gb300.h"
#include "cp3_launch.h"
#include "cp3_tile.cuh"

namespace cp3 {

constexpr int kLLTile = 32;          // energies per table tile of the likelihood tables
constexpr int kLLPerE = 19;          // per (warp, energy): Lambda' (9), Gamma' (9), LL
constexpr int kLLPerL = 11;          // per (warp, energy, layer): T (9), kappa (2)
constexpr int kLLMaxParams = 6 + kMaxRows;
constexpr int kLLFWords = 13;        // float shadow per (energy, layer): T (9), kappa_1, kappa_2 as hi/lo
constexpr int kLLEigWords = 12;      // per (energy, layer): V (9), m (3)

// ------------------------------------------------------------ complex ----
template <class T>
struct Cx {
    T re, im;
};
template <class T>
__device__ __forceinline__ Cx<T> cx(T r, T i) { return Cx<T>{r, i}; }
template <class T>
__device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) { return Cx<T>{a.re + b.re, a.im + b.im}; }
template <class T>
__device__ __forceinline__ Cx<T> operator*(Cx<T> a, Cx<T> b) {
    return Cx<T>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T>
__device__ __forceinline__ Cx<T> operator*(T t, Cx<T> a) { return Cx<T>{t * a.re, t * a.im}; }
template <class T>
__device__ __forceinline__ Cx<T> cj(Cx<T> a) { return Cx<T>{a.re, -a.im}; }
// conj(a) * b
template <class T>
__device__ __forceinline__ Cx<T> cjmul(Cx<T> a, Cx<T> b) {
    return Cx<T>{a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}
// Sums of products in the pair kernel.  FP64 (DFMA-bound): chains of fused
// multiply-adds, the fewest FP64 instructions.  FP32 (bound by latency, not
// by instruction count): products summed in pairs as the plain expressions
// compile (fmul / ffma, then adds), whose rounding errors grow more slowly
// than a chain's where the terms cancel.
__device__ __forceinline__ double fm(double a, double b, double c) { return __fma_rn(a, b, c); }
// s + conj(a) b
__device__ __forceinline__ Cx<double> cjmac(Cx<double> s, Cx<double> a, Cx<double> b) {
    return Cx<double>{fm(a.im, b.im, fm(a.re, b.re, s.re)), fm(-a.im, b.re, fm(a.re, b.im, s.im))};
}
__device__ __forceinline__ Cx<float> cjmac(Cx<float> s, Cx<float> a, Cx<float> b) { return s + cjmul(a, b); }
// s + a b
__device__ __forceinline__ Cx<double> cmac(Cx<double> s, Cx<double> a, Cx<double> b) {
    return Cx<double>{fm(-a.im, b.im, fm(a.re, b.re, s.re)), fm(a.im, b.re, fm(a.re, b.im, s.im))};
}
__device__ __forceinline__ Cx<float> cmac(Cx<float> s, Cx<float> a, Cx<float> b) { return s + a * b; }
// Re(conj(a0) b0 + conj(a1) b1 + conj(a2) b2)
__device__ __forceinline__ double cjdot3_re(Cx<double> a0, Cx<double> b0, Cx<double> a1, Cx<double> b1,
                                            Cx<double> a2, Cx<double> b2) {
    double s = a0.re * b0.re;
    s = fm(a0.im, b0.im, s);
    s = fm(a1.re, b1.re, s);
    s = fm(a1.im, b1.im, s);
    s = fm(a2.re, b2.re, s);
    return fm(a2.im, b2.im, s);
}
__device__ __forceinline__ float cjdot3_re(Cx<float> a0, Cx<float> b0, Cx<float> a1, Cx<float> b1, Cx<float> a2,
                                           Cx<float> b2) {
    return (cjmul(a0, b0) + cjmul(a1, b1) + cjmul(a2, b2)).re;
}
// t0 z0 + t1 z1 + t2 z2 for real t
__device__ __forceinline__ Cx<double> rdot3(double t0, Cx<double> z0, double t1, Cx<double> z1, double t2,
                                            Cx<double> z2) {
    return Cx<double>{fm(t2, z2.re, fm(t1, z1.re, t0 * z0.re)), fm(t2, z2.im, fm(t1, z1.im, t0 * z0.im))};
}
__device__ __forceinline__ Cx<float> rdot3(float t0, Cx<float> z0, float t1, Cx<float> z1, float t2, Cx<float> z2) {
    return t0 * z0 + t1 * z1 + t2 * z2;
}

// One halving step of a many-value warp sum: lanes with bit `off` clear keep
// the first N/2 values and send the second half to their partner, the others
// the reverse; each lane adds what it receives to what it keeps.
template <int N, class T>
__device__ __forceinline__ void warp_halve(T* v, int lane, int off) {
    const bool hi = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < N / 2; i++) {
        const T send = hi ? v[i] : v[i + N / 2];
        const T keep = hi ? v[i + N / 2] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
}

// Sums of 16 values over the warp with 16 shuffles instead of 80 (recursive
// halving): afterwards lanes 2q and 2q + 1 hold the total of value q in v[0].
// A fixed order: deterministic.
template <class T>
__device__ __forceinline__ void warp_sum16(T (&v)[16], int lane) {
    warp_halve<16>(v, lane, 16);
    warp_halve<8>(v, lane, 8);
    warp_halve<4>(v, lane, 4);
    warp_halve<2>(v, lane, 2);
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// The same for 32 values (31 shuffles instead of 160): lane q holds the total
// of value q in v[0].
template <class T>
__device__ __forceinline__ void warp_sum32(T (&v)[32], int lane) {
    warp_halve<32>(v, lane, 16);
    warp_halve<16>(v, lane, 8);
    warp_halve<8>(v, lane, 4);
    warp_halve<4>(v, lane, 2);
    warp_halve<2>(v, lane, 1);
}

// e^{2 pi i t}, t = kappa * L turns; double: the propagate kernels' FP64
// phase (257-entry table, exact reduction, short Taylor series); float:
// double-float product, exact reduction, then FP32 sincospi.
__device__ __forceinline__ Cx<double> phase_of(double kappa, double L, const double2* __restrict__ tab) {
    double c, s;
    phase_f64(kappa, L, tab, c, s);
    return Cx<double>{c, s};
}
__device__ __forceinline__ Cx<float> phase_of(float2 kap, float2 L) {
    const float p = kap.x * L.x;
    float e = fmaf(kap.x, L.x, -p);
    e = fmaf(kap.x, L.y, e);
    e = fmaf(kap.y, L.x, e);
    const float r = (p - rintf(p)) + e;
    float s, c;
    sincospif(2.0f * r, &s, &c);
    return Cx<float>{c, s};
}

struct LLArgs {
    // inputs on the device
    const OscParams* osc;
    const double* cmat;     // [4][3][3]: dH/d(theta12, theta13, dm21, dm32) of H = O diag(0, d1, d2) O^T
    const double* rhoye;    // [nl]
    const double* energies; // [n_en]
    const double* cosines;  // [n_cos]
    const int* maxl;        // [n_cos]
    const double* radii;    // [nl-1]
    const double* flux_e;   // [n_en]
    const double* flux_mu;  // [n_en]
    const double* counts;   // [n_cos][n_en]
    double norm, height_cm;
    int n_cos, n_en, n_en_pad, nl, nl_pad, n_cchunk;
    int anti;
    // tables (FP64, tile kLLTile)
    double* tab;
    double* pe;
    double* len;
    // partials and results
    double* part_l;  // [n_en][nl][n_cchunk][11] (FP64 kernel)
    double* part_e;  // [n_en][n_cchunk][19]
    float* part_l_f; // the same in float for the mixed kernel (null for FP64)
    float* part_e_f;
    // float copies of the inputs for the mixed kernel
    const float* flux_e_f;
    const float* flux_mu_f;
    const float* counts_f;
    float norm_f;
    double* part_g;  // [n_en][7 + n_rows]: per-energy LL and gradient (mapped host memory)
    const int* layer_row;  // [nl]: caller's row of layer l (l >= 1), -1 for layer 0
    int n_rows;
    const double* ye_layer;  // [nl]
    // FP64 eigen-pairs of every (energy, layer) for the reduction
    double* eig;     // [n_en_pad][nl][12]
    // float shadows of the tables for the mixed pair kernel (null for FP64)
    float* tabf;     // tile-major [n_en_pad/32][nl][13][32]
    float* pef;      // [18][n_en_pad]
    float2* lenf;    // [nl_pad][n_cos], hi/lo (layer-major: a warp's 32 cosines are adjacent)
    const double2* ptab;  // 257-entry FP64 phase table (cos, sin of 2 pi j / 256)
    int phase_cache;      // ll_pair_kernel keeps the forward phases in shared memory (ll_pair_cache_bytes)
};

// ---------------------------------------------------------------- prep ----
__global__ void __launch_bounds__(256) ll_prep_kernel(LLArgs a) {
    extern __shared__ double s_v[];
    const int nl = a.nl, eb = blockDim.y;
    const int nbE = (a.n_en_pad + eb - 1) / eb;
    const GridTables g{a.tab, a.pe, a.len, a.n_en_pad, kLLTile, nl, a.nl_pad};
    if ((int)blockIdx.x < nbE) {
        const int l = threadIdx.x, ey = threadIdx.y;
        const int e = blockIdx.x * eb + ey;
        const bool live = (l < nl) && (e < a.n_en_pad);
        double* vme = s_v + ((size_t)ey * nl + (l < nl ? l : 0)) * 9;
        if (a.tabf) {
            // mixed: the double-float eigen-solve (FP32 pipes) writes the float
            // tables the pair kernel reads (T and Lambda'/Gamma' rounded to
            // float, kappa as hi/lo) and the eigen-pairs of the layer kernel;
            // the eigenvectors reach the overlap pass through shared memory as
            // double-float pairs
            const int tile = e / kLLTile, ln = e % kLLTile;
            const bool ok = live && check_ok(kSiteLLPrep, tile, a.n_en_pad / kLLTile);
            float* f = a.tabf + ((size_t)tile * nl + (l < nl ? l : 0)) * kLLFWords * kLLTile + ln;
            if (ok) {
                const double E = a.energies[e < a.n_en ? e : a.n_en - 1];
                const DF Ed = df_from_double(E);
                DF m[3], V[9];
                layer_eigen_df(*a.osc, Ed, df_from_double(a.rhoye[l]), m, V);
                double* ev = a.eig + ((size_t)e * nl + l) * kLLEigWords;
#pragma unroll
                for (int q = 0; q < 9; q++) {
                    ev[q] = df_to_double(V[q]);
                    df_store(vme + q, V[q]);
                }
#pragma unroll
                for (int k = 0; k < 3; k++) ev[9 + k] = df_to_double(m[k]);
                const DF fE = df_rate_factor(Ed);
                const DF k1 = df_mul(df_sub(m[1], m[0]), fE), k2 = df_mul(df_sub(m[2], m[0]), fE);
                f[9 * kLLTile] = k1.hi;
                f[10 * kLLTile] = k1.lo;
                f[11 * kLLTile] = k2.hi;
                f[12 * kLLTile] = k2.lo;
                if (l <= 1) {
                    // Gamma' = columns e, mu of V_0^T W^dagger (l = 0), Lambda' =
                    // rows e, mu of W V_1 (l = 1), W = R23 diag(1, 1, e^{i dcp})
                    const DF c23 = df_load(a.osc->c23_f), s23 = df_load(a.osc->s23_f);
                    const DF s23cd = df_mul(s23, df_load(a.osc->cd_f));
                    DF s23sd = df_mul(s23, df_load(a.osc->sd_f));
                    if (l == 0) s23sd = df_neg(s23sd);
                    const int off = (l == 0) ? 9 : 0;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        a.pef[(size_t)(off + k) * a.n_en_pad + e] = V[k].hi;
                        a.pef[(size_t)(off + 3 + 2 * k) * a.n_en_pad + e] =
                            df_add(df_mul(c23, V[3 + k]), df_mul(s23cd, V[6 + k])).hi;
                        a.pef[(size_t)(off + 4 + 2 * k) * a.n_en_pad + e] = df_mul(s23sd, V[6 + k]).hi;
                    }
                }
            }
            __syncthreads();
            if (ok) {
                // T_l = V_{l+1}^T V_l (the identity for the innermost layer)
                const bool last = !(l + 1 < nl);
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        float t = (i == j) ? 1.0f : 0.0f;
                        if (!last)
                            t = df_add(df_add(df_mul(df_read(vme + 9 + i), df_read(vme + j)),
                                              df_mul(df_read(vme + 12 + i), df_read(vme + 3 + j))),
                                       df_mul(df_read(vme + 15 + i), df_read(vme + 6 + j)))
                                    .hi;
                        f[(3 * i + j) * kLLTile] = t;
                    }
            }
        } else {
            if (live) {
                const double E = a.energies[e < a.n_en ? e : a.n_en - 1];
                double* ev = a.eig + ((size_t)e * nl + l) * kLLEigWords;
                prep_energy_layer<false>(*a.osc, E, a.rhoye[l], l, e, g, vme, ev + 9);
#pragma unroll
                for (int q = 0; q < 9; q++) ev[q] = vme[q];
            }
            __syncthreads();
            if (live) prep_overlap<false>(l, e, g, vme);
        }
    } else {
        // one thread per (cosine, layer)
        const int f = (blockIdx.x - nbE) * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
        const int c = f / a.nl_pad, l = f % a.nl_pad;
        if (c >= a.n_cos) return;
        prep_cosine_layer<false>(a.cosines[c], a.maxl[c], a.radii, a.height_cm, c, l, g);
        if (a.lenf) {
            const double L = a.len[(size_t)c * a.nl_pad + l];
            const float h = f32_rn(L);
            a.lenf[(size_t)l * a.n_cos + c] = make_float2(h, f32_rn(L - f64_of(h)));
        }
    }
}

// ---------------------------------------------------------- pair kernel ----
// Table accessors for energy e (uniform across the warp).
struct LLTab {
    const double* tab;
    const double* pe;
    int e, nl, n_en_pad;
    __device__ __forceinline__ double T(int l, int i, int j) const {
        const int tile = e / kLLTile, lane = e % kLLTile;
        return tab[(((size_t)tile * nl + l) * kFp64Words + 3 * i + j) * kLLTile + lane];
    }
    __device__ __forceinline__ double kap(int l, int k) const {
        const int tile = e / kLLTile, lane = e % kLLTile;
        return tab[(((size_t)tile * nl + l) * kFp64Words + 9 + k) * kLLTile + lane];
    }
    __device__ __forceinline__ double pe_w(int w) const { return pe[(size_t)w * n_en_pad + e]; }
};

// Table source of the pair kernel for energy e and cosine c: FP64 tables for
// the FP64 kernel, their float shadows (kappa and lengths as hi/lo pairs) for
// the mixed kernel, so that its loops hold no FP64 instruction.
template <class R>
struct LLSrc;
template <>
struct LLSrc<double> {
    LLTab tb;
    const double* len;  // this cosine's [nl_pad]
    const double2* ptab;
    __device__ __forceinline__ LLSrc(const LLArgs& a, int e, int c)
        : tb{a.tab, a.pe, e, a.nl, a.n_en_pad}, len(a.len + (size_t)c * a.nl_pad), ptab(a.ptab) {}
    __device__ __forceinline__ double T(int l, int i, int j) const { return tb.T(l, i, j); }
    // e^{i psi_k} of layer l, k = 1, 2 (table words kappa_1, kappa_2)
    __device__ __forceinline__ Cx<double> D(int l, int k) const { return phase_of(tb.kap(l, k - 1), len[l], ptab); }
    __device__ __forceinline__ double L(int l) const { return len[l]; }
    __device__ __forceinline__ double pe(int w) const { return tb.pe_w(w); }
};
template <>
struct LLSrc<float> {
    const float* f;      // this energy's column of layer 0 in the tile-major shadow
    const float* pef;
    const float2* len;   // this cosine's column of the layer-major lengths
    int e, n_en_pad, n_cos;
    __device__ __forceinline__ LLSrc(const LLArgs& a, int e_, int c)
        : f(a.tabf + (size_t)(e_ / kLLTile) * a.nl * kLLFWords * kLLTile + e_ % kLLTile),
          pef(a.pef),
          len(a.lenf + c),
          e(e_),
          n_en_pad(a.n_en_pad),
          n_cos(a.n_cos) {}
    __device__ __forceinline__ float T(int l, int i, int j) const { return f[(l * kLLFWords + 3 * i + j) * kLLTile]; }
    __device__ __forceinline__ Cx<float> D(int l, int k) const {
        const float kh = f[(l * kLLFWords + 7 + 2 * k) * kLLTile], kl = f[(l * kLLFWords + 8 + 2 * k) * kLLTile];
        return phase_of(make_float2(kh, kl), len[(size_t)l * n_cos]);
    }
    __device__ __forceinline__ float L(int l) const { return len[(size_t)l * n_cos].x; }
    __device__ __forceinline__ float pe(int w) const { return pef[(size_t)w * n_en_pad + e]; }
};

// Shared memory of ll_pair_kernel's phase cache: the forward pass's e^{i psi_k}
// of layers 1 .. nl-1, k = 1, 2, for the block's 128 threads, so that the
// backward pass reads them instead of evaluating them again.  Zero (no cache:
// the phases are evaluated twice) where it would cost occupancy: above 56 KB
// per block for the float kernel (4 blocks per SM) and 110 KB for the double
// kernel (2 blocks per SM).
__host__ __device__ inline size_t ll_pair_cache_bytes(bool mixed, int nl) {
    const size_t b = (size_t)nl * 2 * 128 * (mixed ? 2 * sizeof(float) : 2 * sizeof(double));
    return b <= (mixed ? 56u : 110u) * 1024 ? b : 0;
}

template <class R>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 1) ll_pair_kernel(LLArgs a) {
    using C = Cx<R>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + warp;
    const int cchunk = blockIdx.y;
    const int c = cchunk * 32 + lane;
    if (e >= a.n_en) return;  // whole warp leaves together
    if (!check_ok(kSiteLLPair, cchunk, a.n_cchunk)) return;  // the same for the whole block
    const bool valid = c < a.n_cos;
    const int M = valid ? CP3_IX(kSiteLLPair, a.maxl[c], a.nl) : 0;
    const int Mw = __reduce_max_sync(0xffffffffu, M);
    const LLSrc<R> src(a, e, valid ? c : 0);
    const R twopi = (R)kTwoPi;

    // per-energy tables: Lambda' (row 0 real, row 1 complex), Gamma' (col 0 real, col 1 complex)
    R La[3];
    C Lb[3];
    R Ga[3];
    C Gb[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        La[k] = src.pe(k);
        Lb[k] = C{src.pe(3 + 2 * k), src.pe(4 + 2 * k)};
        Ga[k] = src.pe(9 + k);
        Gb[k] = C{src.pe(12 + 2 * k), src.pe(13 + 2 * k)};
    }
    auto T = [&](int l, int i, int j) -> R { return src.T(l, i, j); };
    auto D = [&](int l, int k) -> C { return src.D(l, k); };  // k = 1, 2
    // the forward pass's phases of layers 1 .. M-1, kept for the backward
    // pass when the kernel has the shared memory ([layer][k][thread])
    extern __shared__ __align__(16) unsigned char s_pair_raw[];
    C* s_ph = (C*)s_pair_raw;
    const bool cache = a.phase_cache != 0;
    auto keep = [&](int l, const C d[3]) {
        if (cache) {
            s_ph[((size_t)l * 2 + 0) * blockDim.x + threadIdx.x] = d[1];
            s_ph[((size_t)l * 2 + 1) * blockDim.x + threadIdx.x] = d[2];
        }
    };
    auto Dk = [&](int l, int k) -> C { return cache ? s_ph[((size_t)l * 2 + k - 1) * blockDim.x + threadIdx.x] : D(l, k); };

    // ---------------- forward
    C D0[3] = {C{1, 0}, D(0, 1), D(0, 2)};
    C g[3][2];  // D_0 Gamma'
#pragma unroll
    for (int j = 0; j < 3; j++) {
        g[j][0] = Ga[j] * D0[j];
        g[j][1] = D0[j] * Gb[j];
    }
    C x[3][2];  // T_0 g
    C Y[3][3];
    C DM[3] = {C{1, 0}, C{1, 0}, C{1, 0}};
    C G[3][3];
    C X[3][2];
    C B[2][2];
    if (M >= 1) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int b = 0; b < 2; b++) x[i][b] = rdot3(T(0, i, 0), g[0][b], T(0, i, 1), g[1][b], T(0, i, 2), g[2][b]);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) Y[i][j] = C{(R)(i == j), 0};
        if (M >= 2) {
            // the first eigenstate's phase is 1: its row is not multiplied
            const C d1[3] = {C{1, 0}, D(1, 1), D(1, 2)};
            keep(1, d1);
#pragma unroll
            for (int i = 0; i < 3; i++) {
                Y[i][0] = C{T(1, i, 0), 0};
#pragma unroll
                for (int k = 1; k < 3; k++) Y[i][k] = T(1, i, k) * d1[k];
            }
            for (int l = 2; l < M; l++) {
                const C dl[3] = {C{1, 0}, D(l, 1), D(l, 2)};
                keep(l, dl);
                C U[3][3];
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    U[0][j] = Y[0][j];
#pragma unroll
                    for (int k = 1; k < 3; k++) U[k][j] = dl[k] * Y[k][j];
                }
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) Y[i][j] = rdot3(T(l, i, 0), U[0][j], T(l, i, 1), U[1][j], T(l, i, 2), U[2][j]);
            }
        }
        DM[1] = D(M, 1);
        DM[2] = D(M, 2);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                C s{0, 0};
#pragma unroll
                for (int k = 0; k < 3; k++) s = cmac(s, Y[k][i], DM[k] * Y[k][j]);
                G[i][j] = s;
            }
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int b = 0; b < 2; b++) X[k][b] = cmac(cmac(G[k][0] * x[0][b], G[k][1], x[1][b]), G[k][2], x[2][b]);
#pragma unroll
        for (int b = 0; b < 2; b++) {
            B[0][b] = rdot3(La[0], X[0][b], La[1], X[1][b], La[2], X[2][b]);
            B[1][b] = cmac(cmac(Lb[0] * X[0][b], Lb[1], X[1][b]), Lb[2], X[2][b]);
        }
    } else {
        // block = Gamma'^dagger D_0 Gamma'
#pragma unroll
        for (int b = 0; b < 2; b++) {
            B[0][b] = Ga[0] * g[0][b] + Ga[1] * g[1][b] + Ga[2] * g[2][b];
            B[1][b] = cjmul(Gb[0], g[0][b]) + cjmul(Gb[1], g[1][b]) + cjmul(Gb[2], g[2][b]);
        }
    }
    // probabilities P(e -> mu) = |S[mu][e]|^2 = |B[1][0]|^2, P(mu -> mu) = |B[1][1]|^2;
    // the bin's LL term and its seed in the kernel's precision (the mixed
    // kernel holds no FP64 instruction in its loops)
    const R pem = B[1][0].re * B[1][0].re + B[1][0].im * B[1][0].im;
    const R pmm = B[1][1].re * B[1][1].re + B[1][1].im * B[1][1].im;
    R ll = 0;
    R w_em = 0, w_mm = 0;
    if (valid) {
        R fe, fm, n, nrm;
        if constexpr (std::is_same<R, float>::value) {
            fe = a.flux_e_f[e];
            fm = a.flux_mu_f[e];
            n = a.counts_f[(size_t)c * a.n_en + e];
            nrm = a.norm_f;
        } else {
            fe = a.flux_e[e];
            fm = a.flux_mu[e];
            n = a.counts[(size_t)c * a.n_en + e];
            nrm = a.norm;
        }
        const R lam = nrm * (fe * pem + fm * pmm);
        if (lam > R(0)) {
            ll = n * log(lam) - lam;
            const R w = (n / lam - R(1)) * nrm;
            w_em = w * fe;
            w_mm = w * fm;
        } else {
            ll = -lam;
        }
    }
    // ---------------- backward
    C gB[2][2] = {{C{0, 0}, C{0, 0}}, {(R)2 * w_em * B[1][0], (R)2 * w_mm * B[1][1]}};
    C gLb[3], gGb[3];  // adjoints of Lambda' row 1 and Gamma' column 1
    R gLa[3], gGa[3];
    C gD0[3];
    R gT0[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        gLb[k] = C{0, 0};
        gGb[k] = C{0, 0};
        gLa[k] = 0;
        gGa[k] = 0;
        gD0[k] = C{0, 0};
#pragma unroll
        for (int j = 0; j < 3; j++) gT0[k][j] = 0;
    }
    C gY[3][3];
    C gDM[3] = {C{0, 0}, C{0, 0}, C{0, 0}};
    if (M >= 1) {
        // B = Lambda' X
        C gX[3][2];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int b = 0; b < 2; b++) gX[k][b] = La[k] * gB[0][b] + cjmul(Lb[k], gB[1][b]);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            gLa[k] = (cjmul(X[k][0], gB[0][0]) + cjmul(X[k][1], gB[0][1])).re;
            gLb[k] = cjmul(X[k][0], gB[1][0]) + cjmul(X[k][1], gB[1][1]);
        }
        // X = G x
        C gx[3][2];
        C gG[3][3];
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int b = 0; b < 2; b++) gx[j][b] = cjmul(G[0][j], gX[0][b]) + cjmul(G[1][j], gX[1][b]) + cjmul(G[2][j], gX[2][b]);
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int j = 0; j < 3; j++) gG[k][j] = cjmul(x[j][0], gX[k][0]) + cjmul(x[j][1], gX[k][1]);
        // x = T_0 g
        C gg[3][2];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) gT0[i][j] = (cjmul(g[j][0], gx[i][0]) + cjmul(g[j][1], gx[i][1])).re;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int b = 0; b < 2; b++) gg[j][b] = T(0, 0, j) * gx[0][b] + T(0, 1, j) * gx[1][b] + T(0, 2, j) * gx[2][b];
        // g = D_0 Gamma'
#pragma unroll
        for (int j = 0; j < 3; j++) {
            gD0[j] = (Ga[j] * gg[j][0]) + cjmul(Gb[j], gg[j][1]);
            gGa[j] = cjmul(D0[j], gg[j][0]).re;
            gGb[j] = cjmul(D0[j], gg[j][1]);
        }
        // G = Y^T D_M Y
#pragma unroll
        for (int k = 0; k < 3; k++) {
            C sd{0, 0};
#pragma unroll
            for (int i = 0; i < 3; i++) {
                C s{0, 0};
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    s = cjmac(s, Y[k][j], gG[i][j] + gG[j][i]);
                    sd = cjmac(sd, Y[k][i] * Y[k][j], gG[i][j]);
                }
                gY[k][i] = cjmul(DM[k], s);
            }
            gDM[k] = sd;
        }
    } else {
        // B = Gamma'^dagger g, g = D_0 Gamma'
#pragma unroll
        for (int j = 0; j < 3; j++) {
            // from the left factor: B[0][b] += Ga[j] g[j][b], B[1][b] += conj(Gb[j]) g[j][b]
            gGa[j] = (cjmul(g[j][0], gB[0][0]) + cjmul(g[j][1], gB[0][1])).re;
            gGb[j] = cj(cjmul(g[j][0], gB[1][0]) + cjmul(g[j][1], gB[1][1]));
            C ggj0 = Ga[j] * gB[0][0] + Gb[j] * gB[1][0];
            C ggj1 = Ga[j] * gB[0][1] + Gb[j] * gB[1][1];
            gD0[j] = Ga[j] * ggj0 + cjmul(Gb[j], ggj1);
            gGa[j] += cjmul(D0[j], ggj0).re;
            gGb[j] = gGb[j] + cjmul(D0[j], ggj1);
        }
    }

    // per-(energy, layer) partials: layers Mw .. 1 (descending), then layer 0
    // partials in the kernel's precision (float buffers for the mixed kernel)
    // layout [energy][layer][cosine chunk][11]: a layer's partials are one
    // contiguous block for the layer kernel
    const size_t lstride = (size_t)a.n_cchunk * kLLPerL;
    R* pl = (R*)(std::is_same<R, float>::value ? (void*)a.part_l_f : (void*)a.part_l) +
            (size_t)e * a.nl * lstride + (size_t)cchunk * kLLPerL;
    for (int l = Mw; l >= 1; l--) {
        R tT[9];
        R tk[2] = {0, 0};
#pragma unroll
        for (int q = 0; q < 9; q++) tT[q] = 0;
        if (l == M) {
            // D_M = diag(1, e^{i psi1}, e^{i psi2}): dLL/dkappa_k = 2 pi L * (-Im(conj(gD) D))
#pragma unroll
            for (int k = 1; k < 3; k++) tk[k - 1] = -twopi * src.L(l) * cjmul(gDM[k], DM[k]).im;
        } else if (l < M) {
            // Y_l = T_l U, U = D_l Y_{l-1}; un-multiply: U = T_l^T Y_l, Y_{l-1} = conj(D_l) U
            const C dl[3] = {C{1, 0}, Dk(l, 1), Dk(l, 2)};
            R t[3][3];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) t[i][j] = T(l, i, j);
            C U[3][3], gU[3][3];
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    U[k][j] = rdot3(t[0][k], Y[0][j], t[1][k], Y[1][j], t[2][k], Y[2][j]);
                    gU[k][j] = rdot3(t[0][k], gY[0][j], t[1][k], gY[1][j], t[2][k], gY[2][j]);
                }
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int k = 0; k < 3; k++) tT[3 * i + k] = cjdot3_re(U[k][0], gY[i][0], U[k][1], gY[i][1], U[k][2], gY[i][2]);
            if (l >= 2) {
                // row 0: the first eigenstate's phase is 1
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    Y[0][j] = U[0][j];
                    gY[0][j] = gU[0][j];
                }
#pragma unroll
                for (int k = 1; k < 3; k++) {
                    C gd{0, 0};
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        const C yp = cjmul(dl[k], U[k][j]);  // Y_{l-1}[k][j]
                        gd = cjmac(gd, yp, gU[k][j]);
                        Y[k][j] = yp;
                        gY[k][j] = cjmul(dl[k], gU[k][j]);
                    }
                    tk[k - 1] = -twopi * src.L(l) * cjmul(gd, dl[k]).im;
                }
            } else {
                // l = 1: Y_1 = T_1 D_1, so U = D_1 and gU holds the adjoint of D_1 on the diagonal
#pragma unroll
                for (int k = 1; k < 3; k++) tk[k - 1] = -twopi * src.L(1) * cjmul(gU[k][k], dl[k]).im;
            }
        }
        // warp reduction of this layer's 11 values (lanes with nothing to add
        // give zeros), in the kernel's precision: each term already carries
        // that precision's rounding, a 5-level tree adds at most 5 ulp of the
        // absolute sum
        {
            R v[16];
#pragma unroll
            for (int q = 0; q < 9; q++) v[q] = tT[q];
            v[9] = tk[0];
            v[10] = tk[1];
#pragma unroll
            for (int q = 11; q < 16; q++) v[q] = R(0);
            warp_sum16(v, lane);
            if ((lane & 1) == 0 && (lane >> 1) < kLLPerL) pl[(size_t)l * lstride + (lane >> 1)] = v[0];
        }
    }
    // layers above Mw are never crossed by this warp's cosines
    if (lane == 0)
        for (int l = Mw + 1; l < a.nl; l++)
            for (int q = 0; q < kLLPerL; q++) pl[(size_t)l * lstride + q] = R(0);
    // layer 0: T_0 and D_0
    {
        R v[16];
#pragma unroll
        for (int q = 0; q < 9; q++) v[q] = gT0[q / 3][q % 3];
#pragma unroll
        for (int k = 1; k < 3; k++) v[9 + k - 1] = -twopi * src.L(0) * cjmul(gD0[k], D0[k]).im;
#pragma unroll
        for (int q = 11; q < 16; q++) v[q] = R(0);
        warp_sum16(v, lane);
        if ((lane & 1) == 0 && (lane >> 1) < kLLPerL) pl[lane >> 1] = v[0];
    }
    // per energy: Lambda', Gamma', LL
    R* pe = (R*)(std::is_same<R, float>::value ? (void*)a.part_e_f : (void*)a.part_e) +
            ((size_t)e * a.n_cchunk + cchunk) * kLLPerE;
    R vals[32];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        vals[k] = gLa[k];
        vals[3 + 2 * k] = gLb[k].re;
        vals[4 + 2 * k] = gLb[k].im;
        vals[9 + k] = gGa[k];
        vals[12 + 2 * k] = gGb[k].re;
        vals[13 + 2 * k] = gGb[k].im;
    }
    vals[kLLPerE - 1] = ll;
#pragma unroll
    for (int q = kLLPerE; q < 32; q++) vals[q] = R(0);
    warp_sum32(vals, lane);
    if (lane < kLLPerE) pe[lane] = vals[0];
}

// ---------------------------------------------------------- reduction ----
// Output slots of one energy's gradient row: [0] LL, [1..6] theta12, theta13,
// theta23, dCP, dm12sq, dm23sq, [7 + r] density of the caller's row r.
constexpr int kLLOscOut = 7;

// Items of ll_layer_kernel: (energy slot, row r, layer l), 3 nl per energy,
// packed densely (the FP64 pipe is paid per warp instruction, whatever the
// active lanes), epb energies per block.
__host__ __device__ inline int ll_layer_threads(int nl, int epb) { return (epb * 3 * nl + 31) / 32 * 32; }
__host__ __device__ inline int ll_layer_slot_doubles(int nl) {
    return nl * (9 + 9 + 2 + 3 + 3 + 9) + kLLPerE + 3 * nl * kLLOscOut + 3 * kLLOscOut;
}

// Cosine chunks whose partials ll_layer_kernel loads before summing them.
constexpr int kLLBatch = 8;

// Compensated FP32 sum (Knuth's TwoSum per term): the error of each add is
// carried in c, so s + c is the sum of the float terms to about 2^-46 of their
// magnitudes, on the FP32 pipe instead of float-to-double conversions and FP64
// adds.
struct FloatTwoSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x, bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
    __device__ __forceinline__ double value() const { return f64_of(s) + f64_of(c); }
};

// Item (slot, r, l) of block b: energy b * epb + slot, row r in {0, 1, 2} of
// the 3x3 quantities of layer l, so that the FP64 chain of each (energy,
// layer) is split three ways (the work is 2 x 10^3 short chains, bound by the
// FP64 issue of the busiest SM, not by the GPU's FP64 throughput):
//   1. sums of the warps' partials (11 per layer; the mixed kernel's float
//      partials by compensated FP32 sums), the eigen-pairs solved
//      by the prep kernel and one reciprocal eigenvalue gap per row, into
//      shared memory;
//   2. row r of the eigenvector adjoint gV_l from the two overlaps the layer
//      enters (T_{l-1} = V_l^T V_{l-1}, T_l = V_{l+1}^T V_l) and, for l = 0, 1,
//      from Gamma' / Lambda';
//   3. row r of W, W[j][k] = (v_j . gv_k) / (m_k - m_j) off the diagonal and
//      dLL/dm_k on it (symmetric eigenvector adjoint);
//   4. row r of gH = V W V^T;
//   5. row r's share of the contractions of sym(gH) with the parameter
//      derivatives of H_l = O diag(0, d1, d2) O^T - fac_l e0 e0^T: cmat holds
//      the four symmetrised 3x3 derivative matrices (theta12, theta13, dm21,
//      dm32), formed on the host with the parameters, so the contraction is
//      sum_q gH[r][q] C[r][q].
// Densities map one-to-one to layers (single writer per slot); the
// oscillation parameters of an energy are summed over its items in a fixed
// order (rows' layers, then the three rows).
__global__ void __launch_bounds__(288) ll_layer_kernel(LLArgs a, int epb) {
    extern __shared__ double s_ll[];
    const int nl = a.nl, per = 3 * nl;
    const int slot = threadIdx.x / per, w = threadIdx.x - slot * per;
    const int r = w / nl, l = w - r * nl;
    const int e = blockIdx.x * epb + slot;
    const bool live = slot < epb && e < a.n_en;
    double* sV = s_ll + (size_t)(slot < epb ? slot : 0) * ll_layer_slot_doubles(nl);  // [nl][9]
    double* sT = sV + nl * 9;          // [nl][9] summed adjoint of T_l
    double* sK = sT + nl * 9;          // [nl][2] summed adjoint of kappa_l
    double* sM = sK + nl * 2;          // [nl][3] eigenvalues
    double* sI = sM + nl * 3;          // [nl][3] 1 / (m_{r+1} - m_{r+2}), indices mod 3
    double* sG = sI + nl * 3;          // [nl][9] gV, then W
    double* sL = sG + nl * 9;          // [19]
    double* sAcc = sL + kLLPerE;       // [3 nl][7]
    double* sRow = sAcc + per * kLLOscOut;  // [3][7]
    const OscParams& o = *a.osc;
    const double E = live ? a.energies[e] : 1.0;
    // 1. partial sums, eigen-pairs, reciprocal gaps.  The partials are read
    // kLLBatch chunks at a time with every load of a batch issued before the
    // first add (one memory round trip per batch, not per chunk).
    if (live) {
        const double* ev = a.eig + ((size_t)e * nl + l) * kLLEigWords;
        const int r1 = (r == 2) ? 0 : r + 1, r2 = (r == 0) ? 2 : r - 1;
        double vr[3];
#pragma unroll
        for (int k = 0; k < 3; k++) vr[k] = ev[3 * r + k];
        const double mr = ev[9 + r], m1 = ev[9 + r1], m2 = ev[9 + r2];
        const size_t lb = ((size_t)e * nl + l) * a.n_cchunk * kLLPerL + r;  // this layer's block, q = r
        const int nq = (r < 2) ? 4 : 3;                                    // q = r + 3 i < 11
        double v[4];
        if (a.part_l_f) {
            FloatTwoSum f[4];
            for (int c0 = 0; c0 < a.n_cchunk; c0 += kLLBatch) {
                float x[kLLBatch][4];
#pragma unroll
                for (int u = 0; u < kLLBatch; u++)
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        x[u][i] = (c0 + u < a.n_cchunk && i < nq) ? a.part_l_f[lb + (size_t)(c0 + u) * kLLPerL + 3 * i] : 0.0f;
#pragma unroll
                for (int u = 0; u < kLLBatch; u++)
#pragma unroll
                    for (int i = 0; i < 4; i++) f[i].add(x[u][i]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++) v[i] = f[i].value();
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) v[i] = 0.0;
            for (int c0 = 0; c0 < a.n_cchunk; c0 += kLLBatch) {
                double x[kLLBatch][4];
#pragma unroll
                for (int u = 0; u < kLLBatch; u++)
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        x[u][i] = (c0 + u < a.n_cchunk && i < nq) ? a.part_l[lb + (size_t)(c0 + u) * kLLPerL + 3 * i] : 0.0;
#pragma unroll
                for (int u = 0; u < kLLBatch; u++)
#pragma unroll
                    for (int i = 0; i < 4; i++) v[i] += x[u][i];
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int q = r + 3 * i;
            if (q < 9)
                sT[l * 9 + q] = v[i];
            else if (q < kLLPerL)
                sK[l * 2 + q - 9] = v[i];
        }
#pragma unroll
        for (int k = 0; k < 3; k++) sV[l * 9 + 3 * r + k] = vr[k];
        sM[l * 3 + r] = mr;
        const double gap = m1 - m2;
        sI[l * 3 + r] = (gap != 0.0) ? 1.0 / gap : 0.0;
        for (int q = w; q < kLLPerE; q += per) {
            const size_t pb = (size_t)e * a.n_cchunk * kLLPerE + q;
            double sum = 0.0;
            if (a.part_e_f) {
                FloatTwoSum f;
                for (int c0 = 0; c0 < a.n_cchunk; c0 += kLLBatch) {
                    float x[kLLBatch];
#pragma unroll
                    for (int u = 0; u < kLLBatch; u++) x[u] = (c0 + u < a.n_cchunk) ? a.part_e_f[pb + (size_t)(c0 + u) * kLLPerE] : 0.0f;
#pragma unroll
                    for (int u = 0; u < kLLBatch; u++) f.add(x[u]);
                }
                sum = f.value();
            } else {
                for (int c0 = 0; c0 < a.n_cchunk; c0 += kLLBatch) {
                    double x[kLLBatch];
#pragma unroll
                    for (int u = 0; u < kLLBatch; u++) x[u] = (c0 + u < a.n_cchunk) ? a.part_e[pb + (size_t)(c0 + u) * kLLPerE] : 0.0;
#pragma unroll
                    for (int u = 0; u < kLLBatch; u++) sum += x[u];
                }
            }
            sL[q] = sum;
        }
    }
    __syncthreads();

    double acc[kLLOscOut];
#pragma unroll
    for (int q = 0; q < kLLOscOut; q++) acc[q] = 0.0;
    // 2. row r of gV_l
    if (live) {
        double gvr[3] = {0.0, 0.0, 0.0};
        // T_l = V_{l+1}^T V_l: dT_l[i][c] / dV_l[r][c] = V_{l+1}[r][i]
        if (l + 1 < nl)
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int i = 0; i < 3; i++) gvr[c] += sT[l * 9 + 3 * i + c] * sV[(l + 1) * 9 + 3 * r + i];
        // T_{l-1} = V_l^T V_{l-1}: dT_{l-1}[c][j] / dV_l[r][c] = V_{l-1}[r][j]
        if (l >= 1)
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int j = 0; j < 3; j++) gvr[c] += sT[(l - 1) * 9 + 3 * c + j] * sV[(l - 1) * 9 + 3 * r + j];
        if (l <= 1) {
            // l = 1, Lambda' from V_1: row 0 = V_1[0][k]; row 1 = c23 V_1[1][k] + s23 e^{i d} V_1[2][k]
            // l = 0, Gamma' from V_0: column 0 = V_0[0][k]; column 1 = c23 V_0[1][k] + s23 e^{-i d} V_0[2][k]
            const double s23 = o.s23, c23 = o.c23, sd = o.sd, cd = o.cd;
            const int off = (l == 1) ? 0 : 9;
            const double sg = (l == 1) ? 1.0 : -1.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const double gre = sL[off + 3 + 2 * k], gim = sL[off + 4 + 2 * k];
                if (r == 0) gvr[k] += sL[off + k];
                if (r == 1) gvr[k] += c23 * gre;
                if (r == 2) gvr[k] += s23 * (gre * cd + sg * gim * sd);
                if (r == 0) {
                    const double v1 = sV[l * 9 + 3 + k], v2 = sV[l * 9 + 6 + k];
                    // d/dtheta23: -s23 v1 + c23 e^{+-id} v2 ; d/ddcp: +-i s23 e^{+-id} v2
                    acc[3] += gre * (-s23 * v1 + c23 * cd * v2) + gim * (sg * c23 * sd * v2);
                    acc[4] += gre * (-s23 * sd * v2) + gim * (sg * s23 * cd * v2);
                }
            }
            if (l == 0 && r == 0) acc[0] = sL[18];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) sG[l * 9 + 3 * r + c] = gvr[c];
    }
    __syncthreads();
    // 3. row j = r of W; 1 / (m_k - m_r) = +-sI[t], t the third index
    double wr[3];
    if (live) {
        const double f = phase_rate_factor(E);
        const double gK0 = sK[l * 2], gK1 = sK[l * 2 + 1];
        const double gm[3] = {-(gK0 + gK1) * f, gK0 * f, gK1 * f};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (k == r) {
                wr[k] = gm[k];
            } else {
                double dot = 0.0;
#pragma unroll
                for (int q = 0; q < 3; q++) dot += sV[l * 9 + 3 * q + r] * sG[l * 9 + 3 * q + k];
                const int t = 3 - k - r;
                const double inv = sI[l * 3 + t];
                wr[k] = dot * (((t == 2 ? 0 : t + 1) == k) ? inv : -inv);
            }
        }
    }
    __syncthreads();
    if (live)
#pragma unroll
        for (int k = 0; k < 3; k++) sG[l * 9 + 3 * r + k] = wr[k];
    __syncthreads();
    if (live) {
        // 4. row p = r of gH = V W V^T: u_k = sum_j V[r][j] W[j][k], gH[r][q] = sum_k u_k V[q][k]
        double u[3] = {0.0, 0.0, 0.0}, hr[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int j = 0; j < 3; j++) u[k] += sV[l * 9 + 3 * r + j] * sG[l * 9 + 3 * j + k];
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int k = 0; k < 3; k++) hr[q] += u[k] * sV[l * 9 + 3 * q + k];
        // 5. contractions of row r of gH with the symmetrised derivative matrices
        const double* C = a.cmat + 3 * r;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            acc[1] += hr[q] * C[q];
            acc[2] += hr[q] * C[9 + q];
            acc[5] += hr[q] * C[18 + q];
            acc[6] += hr[q] * C[27 + q];
        }
        // densities: H[0][0] -= fac, fac = sgn GF E rho Ye
        if (l >= 1 && r == 0) {
            const double sgn = a.anti ? 1.0 : -1.0;
            const int np = 6 + a.n_rows;
            a.part_g[(size_t)e * (1 + np) + 1 + 6 + CP3_IX(kSiteLLLayer, a.layer_row[l], a.n_rows)] =
                -hr[0] * sgn * kGF * E * a.ye_layer[l];
        }
#pragma unroll
        for (int q = 0; q < kLLOscOut; q++) sAcc[w * kLLOscOut + q] = acc[q];
    }
    __syncthreads();
    // fixed-order sums of each energy's items: the layers of a row, then the rows
    if (live)
        for (int t = w; t < 3 * kLLOscOut; t += per) {
            const int q = t % kLLOscOut, rr = t / kLLOscOut;
            double v = 0.0;
            for (int i = 0; i < nl; i++) v += sAcc[(rr * nl + i) * kLLOscOut + q];
            sRow[rr * kLLOscOut + q] = v;
        }
    __syncthreads();
    if (live)
        for (int t = w; t < kLLOscOut; t += per)
            a.part_g[(size_t)e * (7 + a.n_rows) + t] = (sRow[t] + sRow[kLLOscOut + t]) + sRow[2 * kLLOscOut + t];
}

}  // namespace cp3

// ======================================================================= host
namespace {

int lfail(int code, const std::string& m) {
    cp3::set_last_error(m);
    return code;
}
int lcuda(cudaError_t e, const char* w) { return lfail(CP3_ERR_CUDA, std::string(w) + ": " + cudaGetErrorString(e)); }

struct LGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit LGuard(int d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) err = cudaSetDevice(d);
    }
    ~LGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

struct cp3_loglik {
    int device = 0;
    bool mixed = false;
    int n_cos = 0, n_en = 0;
    std::vector<double> cosines, energies, flux_e, flux_mu, counts;
    std::vector<int> maxl;
    std::vector<double> radii, ye, coslimit;  // outside-in
    std::vector<int> layer_row;               // caller row of each layer
    int n_rows = 0;
    double height_cm = 0, norm = 1;
    bool has_bins = false, has_body = false, has_flux = false, has_counts = false, has_height = false;
    bool dirty = true;
    int nl = 0, nl_pad = 0, n_en_pad = 0, n_cchunk = 0;
    cudaStream_t stream = nullptr;
    // device
    double *d_en = nullptr, *d_cos = nullptr, *d_radii = nullptr, *d_fe = nullptr, *d_fm = nullptr, *d_counts = nullptr;
    double *d_tab = nullptr, *d_pe = nullptr, *d_len = nullptr, *d_pl = nullptr, *d_pee = nullptr;
    float *d_plf = nullptr, *d_peef = nullptr, *d_fef = nullptr, *d_fmf = nullptr, *d_cntf = nullptr;
    double* d_eig = nullptr;
    float *d_tabf = nullptr, *d_pef = nullptr;
    float2* d_lenf = nullptr;
    int4* d_ptab = nullptr;
    double* d_yel = nullptr;
    int *d_maxl = nullptr, *d_row = nullptr;
    cp3::OscParams* d_osc = nullptr;
    // pinned staging [OscParams, cmat][rhoye], uploaded by one copy into d_osc;
    // h_rows is mapped [n_en][7 + n_rows]: ll_layer_kernel writes each
    // energy's log-likelihood and gradient terms there directly
    unsigned char* h_up = nullptr;
    double* h_rows = nullptr;
    double* dh_rows = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_type = -1;
    // optional kernel timing: events recorded by the graph before the prep
    // kernel and after each of the three kernels
    bool timing = false;
    bool timed = false;  // the last evaluation ran a graph with the events
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace {

void ll_free(cp3_loglik* L) {
    if (L->exec) cudaGraphExecDestroy(L->exec);
    if (L->graph) cudaGraphDestroy(L->graph);
    L->exec = nullptr;
    L->graph = nullptr;
    void* ptrs[] = {L->d_en, L->d_cos, L->d_radii, L->d_fe, L->d_fm, L->d_counts, L->d_tab, L->d_pe, L->d_len,
                    L->d_pl, L->d_pee, L->d_yel, L->d_maxl, L->d_row, L->d_osc,
                    L->d_eig, L->d_tabf, L->d_pef, L->d_lenf, L->d_plf, L->d_peef, L->d_fef, L->d_fmf, L->d_cntf,
                    L->d_ptab};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    L->d_en = L->d_cos = L->d_radii = L->d_fe = L->d_fm = L->d_counts = nullptr;
    L->d_tab = L->d_pe = L->d_len = L->d_pl = L->d_pee = L->d_yel = nullptr;
    L->d_eig = nullptr;
    L->d_tabf = L->d_pef = nullptr;
    L->d_lenf = nullptr;
    L->d_ptab = nullptr;
    L->d_plf = L->d_peef = L->d_fef = L->d_fmf = L->d_cntf = nullptr;
    L->d_maxl = L->d_row = nullptr;
    L->d_osc = nullptr;
}

// Parameter block uploaded by the graph's first copy: OscParams, then the four
// 3x3 derivative matrices of the vacuum Hamiltonian at kCmatOff.
constexpr size_t kCmatOff = (sizeof(cp3::OscParams) + 15) / 16 * 16;
constexpr size_t kOscBlock = kCmatOff + 36 * sizeof(double);

constexpr size_t kUpBytes = kOscBlock + sizeof(double) * (cp3::kMaxRows + 1);

template <class T>
cudaError_t dmalloc_copy(T** d, const T* h, size_t n) {
    cudaError_t e = cudaMalloc((void**)d, std::max<size_t>(n, 1) * sizeof(T));
    if (!e && n) e = cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

cp3::LLArgs ll_args(cp3_loglik* L, int type) {
    cp3::LLArgs a{};
    a.osc = L->d_osc;
    a.cmat = (const double*)((const unsigned char*)L->d_osc + kCmatOff);
    a.rhoye = (const double*)((const unsigned char*)L->d_osc + kOscBlock);
    a.energies = L->d_en;
    a.cosines = L->d_cos;
    a.maxl = L->d_maxl;
    a.radii = L->d_radii;
    a.flux_e = L->d_fe;
    a.flux_mu = L->d_fm;
    a.counts = L->d_counts;
    a.norm = L->norm;
    a.height_cm = L->height_cm;
    a.n_cos = L->n_cos;
    a.n_en = L->n_en;
    a.n_en_pad = L->n_en_pad;
    a.nl = L->nl;
    a.nl_pad = L->nl_pad;
    a.n_cchunk = L->n_cchunk;
    a.anti = type == CP3_ANTINEUTRINO;
    a.tab = L->d_tab;
    a.pe = L->d_pe;
    a.len = L->d_len;
    a.part_l = L->d_pl;
    a.part_e = L->d_pee;
    a.part_g = L->dh_rows;
    a.eig = L->d_eig;
    a.tabf = L->mixed ? L->d_tabf : nullptr;
    a.pef = L->mixed ? L->d_pef : nullptr;
    a.lenf = L->mixed ? L->d_lenf : nullptr;
    a.ptab = (const double2*)L->d_ptab;
    a.phase_cache = cp3::ll_pair_cache_bytes(L->mixed, L->nl) > 0;
    a.part_l_f = L->mixed ? L->d_plf : nullptr;
    a.part_e_f = L->mixed ? L->d_peef : nullptr;
    a.flux_e_f = L->d_fef;
    a.flux_mu_f = L->d_fmf;
    a.counts_f = L->d_cntf;
    a.norm_f = (float)L->norm;
    a.layer_row = L->d_row;
    a.n_rows = L->n_rows;
    a.ye_layer = L->d_yel;
    return a;
}

// Device buffers and the evaluation graph: upload, prep, pairs, reduce, download.
int ll_setup(cp3_loglik* L, int type) {
    ll_free(L);
    L->nl = L->n_rows + 1;
    L->nl_pad = (L->nl + 1) / 2 * 2;
    L->n_en_pad = (L->n_en + cp3::kLLTile - 1) / cp3::kLLTile * cp3::kLLTile;
    L->n_cchunk = (L->n_cos + 31) / 32;
    for (int i = 0; i < L->n_cos; i++) {
        int cnt = 0;
        for (double lim : L->coslimit) cnt += (L->cosines[i] < lim);
        L->maxl[i] = cnt;
    }
    std::vector<double> yel(L->nl, 0.0);
    for (int l = 1; l < L->nl; l++) yel[l] = L->ye[l - 1];
    cudaError_t e;
    if ((e = dmalloc_copy(&L->d_en, L->energies.data(), L->n_en)) || (e = dmalloc_copy(&L->d_cos, L->cosines.data(), L->n_cos)) ||
        (e = dmalloc_copy(&L->d_radii, L->radii.data(), L->radii.size())) ||
        (e = dmalloc_copy(&L->d_fe, L->flux_e.data(), L->n_en)) || (e = dmalloc_copy(&L->d_fm, L->flux_mu.data(), L->n_en)) ||
        (e = dmalloc_copy(&L->d_counts, L->counts.data(), L->counts.size())) ||
        (e = dmalloc_copy(&L->d_maxl, L->maxl.data(), L->n_cos)) ||
        (e = dmalloc_copy(&L->d_row, L->layer_row.data(), L->layer_row.size())) ||
        (e = dmalloc_copy(&L->d_yel, yel.data(), yel.size())))
        return lcuda(e, "loglik inputs");
    const size_t tab = (size_t)L->n_en_pad * L->nl * cp3::kFp64Words, pe = (size_t)cp3::kPerEWords * L->n_en_pad;
    const size_t len = (size_t)L->n_cos * L->nl_pad;
    const size_t pl = (size_t)L->n_cchunk * L->n_en * L->nl * cp3::kLLPerL;
    const size_t pee = (size_t)L->n_cchunk * L->n_en * cp3::kLLPerE;
    if ((e = cudaMalloc(&L->d_tab, tab * 8)) || (e = cudaMalloc(&L->d_pe, pe * 8)) || (e = cudaMalloc(&L->d_len, len * 8)) ||
        (e = cudaMalloc(&L->d_pl, pl * 8)) || (e = cudaMalloc(&L->d_pee, pee * 8)) ||
        (e = cudaMalloc((void**)&L->d_osc, kUpBytes)) ||
        (e = cudaMalloc(&L->d_eig, (size_t)L->n_en_pad * L->nl * cp3::kLLEigWords * 8)))
        return lcuda(e, "cudaMalloc(loglik)");
    {
        std::vector<int4> ptab(cp3::kPhaseTabN + 1);
        cp3::fill_phase_table(false, ptab.data());
        if ((e = dmalloc_copy(&L->d_ptab, ptab.data(), ptab.size()))) return lcuda(e, "loglik phase table");
    }
    if (L->mixed) {
        std::vector<float> fe(L->flux_e.begin(), L->flux_e.end()), fm(L->flux_mu.begin(), L->flux_mu.end());
        std::vector<float> cnt(L->counts.begin(), L->counts.end());
        if ((e = dmalloc_copy(&L->d_fef, fe.data(), fe.size())) || (e = dmalloc_copy(&L->d_fmf, fm.data(), fm.size())) ||
            (e = dmalloc_copy(&L->d_cntf, cnt.data(), cnt.size())) || (e = cudaMalloc(&L->d_plf, pl * 4)) ||
            (e = cudaMalloc(&L->d_peef, pee * 4)))
            return lcuda(e, "cudaMalloc(loglik)");
    }
    if (L->mixed &&
        ((e = cudaMalloc(&L->d_tabf, (size_t)L->n_en_pad * L->nl * cp3::kLLFWords * 4)) ||
         (e = cudaMalloc(&L->d_pef, (size_t)18 * L->n_en_pad * 4)) || (e = cudaMalloc(&L->d_lenf, len * 8))))
        return lcuda(e, "cudaMalloc(loglik)");
    // the pair kernel's phase cache may take more than the default 48 KB of
    // dynamic shared memory (opted in per device, before the capture)
    const size_t pair_smem = cp3::ll_pair_cache_bytes(L->mixed, L->nl);
    if (pair_smem > 48 * 1024 &&
        (e = cp3::opt_in_max_smem(L->mixed ? (const void*)cp3::ll_pair_kernel<float> : (const void*)cp3::ll_pair_kernel<double>)))
        return lcuda(e, "cudaFuncSetAttribute(ll_pair_kernel)");
    // capture
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking))) return lcuda(e, "cudaStreamCreate");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const cp3::LLArgs a = ll_args(L, type);
    if (!e) e = cudaMemcpyAsync(L->d_osc, L->h_up, kOscBlock + sizeof(double) * L->nl, cudaMemcpyHostToDevice, cs);
    // event-record nodes around the kernels when timing is on
    auto stamp = [&](int k) {
        if (!e && L->timing) e = cudaEventRecordWithFlags(L->ev[k], cs, cudaEventRecordExternal);
    };
    stamp(0);
    if (!e) {
        // energies per prep block: enough blocks to spread the FP64
        // eigen-solves over the GPU (about two per SM), at most 256 threads
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, L->device);
        const int eb = std::max(1, std::min(256 / L->nl, std::max(32 / L->nl, L->n_en_pad / std::max(1, 2 * sms))));
        const int nbE = (L->n_en_pad + eb - 1) / eb;
        const int nbC = (L->n_cos * L->nl_pad + L->nl * eb - 1) / (L->nl * eb);
        cp3::ll_prep_kernel<<<nbE + nbC, dim3(L->nl, eb), (size_t)eb * L->nl * 9 * 8, cs>>>(a);
        e = cudaGetLastError();
    }
    stamp(1);
    if (!e) {
        dim3 grid((L->n_en + 3) / 4, L->n_cchunk);
        if (L->mixed)
            cp3::ll_pair_kernel<float><<<grid, 128, pair_smem, cs>>>(a);
        else
            cp3::ll_pair_kernel<double><<<grid, 128, pair_smem, cs>>>(a);
        e = cudaGetLastError();
    }
    stamp(2);
    if (!e) {
        // energies per block: the fewest warps on the busiest SM (the
        // kernel is bound by the FP64 issue of that SM), at most 288 threads
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, L->device);
        sms = std::max(sms, 1);
        int epb = 1;
        long best = -1;
        for (int k = 1; k <= std::max(1, 288 / (3 * L->nl)); k++) {
            const long blocks = (L->n_en + k - 1) / k;
            const long cost = (blocks + sms - 1) / sms * (cp3::ll_layer_threads(L->nl, k) / 32);
            if (best < 0 || cost < best) best = cost, epb = k;
        }
        const int threads = cp3::ll_layer_threads(L->nl, epb);
        const size_t smem = (size_t)epb * cp3::ll_layer_slot_doubles(L->nl) * 8;
        cp3::ll_layer_kernel<<<(L->n_en + epb - 1) / epb, threads, smem, cs>>>(a, epb);
        e = cudaGetLastError();
    }
    stamp(3);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (e || e2) {
        if (g) cudaGraphDestroy(g);
        return lcuda(e ? e : e2, "loglik graph capture");
    }
    L->graph = g;
    if ((e = cudaGraphInstantiate(&L->exec, g, 0))) return lcuda(e, "cudaGraphInstantiate");
    L->graph_type = type;
    L->dirty = false;
    L->timed = L->timing;
    return CP3_OK;
}

}  // namespace

extern "C" {

int cp3_loglik_create(cp3_loglik** out, int device_id, int precision, int n_cos, int n_en) {
    if (!out) return lfail(CP3_ERR_ARGUMENT, "cp3_loglik_create: null output pointer");
    *out = nullptr;
    if (n_cos <= 0 || n_en <= 0) return lfail(CP3_ERR_ARGUMENT, "cp3_loglik_create: empty binning");
    if (precision != CP3_PRECISION_FP64 && precision != CP3_PRECISION_MIXED)
        return lfail(CP3_ERR_ARGUMENT, "cp3_loglik_create: unknown precision");
    if (device_id < 0 || device_id >= cp3_device_count()) return lfail(CP3_ERR_NO_DEVICE, "No GPU found");
    LGuard g(device_id);
    if (g.err) return lcuda(g.err, "cudaSetDevice");
    cp3_loglik* L = new cp3_loglik();
    L->device = device_id;
    L->mixed = precision == CP3_PRECISION_MIXED;
    L->n_cos = n_cos;
    L->n_en = n_en;
    L->maxl.assign(n_cos, 0);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking)) ||
        (e = cudaMallocHost((void**)&L->h_up, kUpBytes)) ||
        (e = cudaHostAlloc((void**)&L->h_rows, sizeof(double) * (size_t)n_en * (cp3::kLLMaxParams + 1),
                           cudaHostAllocMapped)) ||
        (e = cudaHostGetDevicePointer((void**)&L->dh_rows, L->h_rows, 0))) {
        int rc = lcuda(e, "loglik create");
        cp3_loglik_destroy(L);
        return rc;
    }
    *out = L;
    return CP3_OK;
}

int cp3_loglik_destroy(cp3_loglik* L) {
    if (!L) return CP3_OK;
    LGuard g(L->device);
    if (L->stream) cudaStreamSynchronize(L->stream);
    ll_free(L);
    for (cudaEvent_t ev : L->ev)
        if (ev) cudaEventDestroy(ev);
    if (L->h_up) cudaFreeHost(L->h_up);
    if (L->h_rows) cudaFreeHost(L->h_rows);
    if (L->stream) cudaStreamDestroy(L->stream);
    delete L;
    return CP3_OK;
}

int cp3_loglik_set_bins(cp3_loglik* L, const double* cosines, const double* energies) {
    if (!L || !cosines || !energies) return lfail(CP3_ERR_ARGUMENT, "null argument");
    for (int i = 0; i < L->n_cos; i++)
        if (!(cosines[i] >= -1.0 && cosines[i] <= 1.0)) return lfail(CP3_ERR_ARGUMENT, "cosines must lie in [-1, 1]");
    for (int i = 0; i < L->n_en; i++)
        if (!(energies[i] > 0.0) || !std::isfinite(energies[i]))
            return lfail(CP3_ERR_ARGUMENT, "energies must be finite and positive");
    L->cosines.assign(cosines, cosines + L->n_cos);
    L->energies.assign(energies, energies + L->n_en);
    L->has_bins = true;
    L->dirty = true;
    return CP3_OK;
}

int cp3_loglik_set_body(cp3_loglik* L, const double* radii, const double* ye, int n) {
    if (!L || !radii || n <= 0) return lfail(CP3_ERR_ARGUMENT, "setDensity : vectors must not be empty");
    if (n > CP3_MAX_ROWS) return lfail(CP3_ERR_LIMIT, "setDensity : more than 64 rows");
    // the single-grid handle's ordering and checks (propagator.hpp:117-161);
    // the densities are parameters of the evaluation, so none are given here
    const double no_rhos[CP3_MAX_ROWS] = {};
    cp3::BodyRow rows[CP3_MAX_ROWS];
    if (const char* msg = cp3::order_body(radii, no_rhos, ye, n, rows)) return lfail(CP3_ERR_ARGUMENT, msg);
    L->radii.resize(n);
    L->ye.resize(n);
    L->coslimit.resize(n);
    L->layer_row.assign(n + 1, -1);
    for (int i = 0; i < n; i++) {
        L->radii[i] = rows[i].radius;
        L->ye[i] = rows[i].ye;
        L->coslimit[i] = rows[i].coslimit;
        L->layer_row[i + 1] = rows[i].row;
    }
    L->n_rows = n;
    L->has_body = true;
    L->dirty = true;
    return CP3_OK;
}

int cp3_loglik_set_production_height(cp3_loglik* L, double km) {
    if (!L || !std::isfinite(km)) return lfail(CP3_ERR_ARGUMENT, "setProductionHeight: height must be finite");
    L->height_cm = km * 100000.0;
    L->has_height = true;
    L->dirty = true;
    return CP3_OK;
}

int cp3_loglik_set_flux(cp3_loglik* L, const double* flux_e, const double* flux_mu, double norm) {
    if (!L || !flux_e || !flux_mu || !std::isfinite(norm)) return lfail(CP3_ERR_ARGUMENT, "bad flux");
    L->flux_e.assign(flux_e, flux_e + L->n_en);
    L->flux_mu.assign(flux_mu, flux_mu + L->n_en);
    L->norm = norm;
    L->has_flux = true;
    L->dirty = true;
    return CP3_OK;
}

int cp3_loglik_set_observed(cp3_loglik* L, const double* counts) {
    if (!L || !counts) return lfail(CP3_ERR_ARGUMENT, "null counts");
    L->counts.assign(counts, counts + (size_t)L->n_cos * L->n_en);
    L->has_counts = true;
    L->dirty = true;
    return CP3_OK;
}

int cp3_loglik_evaluate(cp3_loglik* L, int type, const double* params, const double* rhos, double* loglik,
                        double* grad) {
    if (!L || !params || !rhos) return lfail(CP3_ERR_ARGUMENT, "null argument");
    if (!L->has_bins || !L->has_body || !L->has_flux || !L->has_counts || !L->has_height)
        return lfail(CP3_ERR_STATE, "loglik: bins, body, flux, observed counts and production height must be set");
    if (type != CP3_NEUTRINO && type != CP3_ANTINEUTRINO) return lfail(CP3_ERR_ARGUMENT, "unknown neutrino type");
    for (int k = 0; k < 6; k++)
        if (!std::isfinite(params[k])) return lfail(CP3_ERR_ARGUMENT, "loglik: parameters must be finite");
    for (int r = 0; r < L->n_rows; r++)
        if (!(rhos[r] >= 0.0)) return lfail(CP3_ERR_ARGUMENT, "loglik: densities must be >= 0");
    LGuard g(L->device);
    cudaGetLastError();  // a failed earlier call must not be reported below
    if (L->dirty || type != L->graph_type) {
        if (int rc = ll_setup(L, type)) return rc;
    }
    // parameters into the pinned staging buffer (read by the graph's first copies)
    cp3::OscParams o{};
    cp3::fill_osc_params(o, params[0], params[1], params[2], params[3], params[4], params[5], type == CP3_ANTINEUTRINO);
    {
        const double s12 = std::sin(params[0]), c12 = std::cos(params[0]);
        const double s13 = std::sin(params[1]), c13 = std::cos(params[1]);
        const double* O = o.o;
        // dH/dp of H = O diag(0, d1, d2) O^T (d1 = dm21, d2 = dm21 + dm32):
        // theta_ij through O (dO D O^T + O D dO^T), the splittings through
        // the outer products of O's columns
        const double dO12[9] = {-c13 * s12, c13 * c12, 0.0, -c12, -s12, 0.0, s13 * s12, -s13 * c12, 0.0};
        const double dO13[9] = {-s13 * c12, -s13 * s12, c13, 0.0, 0.0, 0.0, -c13 * c12, -c13 * s12, -s13};
        const double dd[3] = {0.0, o.d1, o.d2};
        double* C = (double*)(L->h_up + kCmatOff);
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) {
                double t12 = 0.0, t13 = 0.0;
                for (int k = 1; k < 3; k++) {
                    t12 += dd[k] * (dO12[3 * r + k] * O[3 * q + k] + O[3 * r + k] * dO12[3 * q + k]);
                    t13 += dd[k] * (dO13[3 * r + k] * O[3 * q + k] + O[3 * r + k] * dO13[3 * q + k]);
                }
                const double a1 = O[3 * r + 1] * O[3 * q + 1], a2 = O[3 * r + 2] * O[3 * q + 2];
                C[3 * r + q] = t12;
                C[9 + 3 * r + q] = t13;
                C[18 + 3 * r + q] = a1 + a2;
                C[27 + 3 * r + q] = a2;
            }
    }
    std::memcpy(L->h_up, &o, sizeof o);
    double* rhoye = (double*)(L->h_up + kOscBlock);
    rhoye[0] = 0.0;
    for (int l = 1; l < L->nl; l++) rhoye[l] = rhos[L->layer_row[l]] * L->ye[l - 1];
    cudaError_t e = cudaGraphLaunch(L->exec, L->stream);
    if (!e) e = cudaStreamSynchronize(L->stream);
    if (e) return lcuda(e, "loglik evaluation");
    if (cp3::kChecked) {  // the bounds-checked build reports failed checks of this evaluation
        cp3::CheckRecord r{};
        if ((e = cp3::check_take(&r))) return lcuda(e, "bounds-check record");
        if (int rc = cp3::check_status(r)) return rc;
    }
    // fixed-order sums of the energies' rows (slot 0 the log-likelihood, then
    // the 6 oscillation parameters and the density rows)
    const int np1 = 7 + L->n_rows;
    double s[cp3::kLLMaxParams + 1] = {};
    for (int en = 0; en < L->n_en; en++) {
        const double* row = L->h_rows + (size_t)en * np1;
        for (int q = 0; q < np1; q++) s[q] += row[q];
    }
    if (loglik) *loglik = s[0];
    if (grad)
        for (int q = 0; q < 6 + L->n_rows; q++) grad[q] = s[1 + q];
    return CP3_OK;
}

int cp3_loglik_set_kernel_timing(cp3_loglik* L, int enable) {
    if (!L) return lfail(CP3_ERR_ARGUMENT, "null argument");
    LGuard g(L->device);
    if (g.err) return lcuda(g.err, "cudaSetDevice");
    if (enable && !L->ev[0])
        for (cudaEvent_t& ev : L->ev) {
            cudaError_t e = cudaEventCreate(&ev);
            if (e) return lcuda(e, "cudaEventCreate");
        }
    if ((enable != 0) != L->timing) L->dirty = true;  // the graph is captured again with or without the events
    L->timing = enable != 0;
    return CP3_OK;
}

int cp3_loglik_last_kernel_ms(cp3_loglik* L, float* prep_ms, float* pair_ms, float* layer_ms) {
    if (!L) return lfail(CP3_ERR_ARGUMENT, "null argument");
    if (!L->timed || !L->exec) return lfail(CP3_ERR_STATE, "loglik_last_kernel_ms: no timed evaluation");
    LGuard g(L->device);
    float t[3] = {0, 0, 0};
    cudaError_t e = cudaEventSynchronize(L->ev[3]);
    for (int k = 0; k < 3 && !e; k++) e = cudaEventElapsedTime(&t[k], L->ev[k], L->ev[k + 1]);
    if (e) return lcuda(e, "cudaEventElapsedTime");
    if (prep_ms) *prep_ms = t[0];
    if (pair_ms) *pair_ms = t[1];
    if (layer_ms) *layer_ms = t[2];
    return CP3_OK;
}

int cp3_loglik_io_bytes(cp3_loglik* L, long long* host_to_device, long long* device_to_host) {
    if (!L) return lfail(CP3_ERR_ARGUMENT, "null argument");
    if (!L->has_body) return lfail(CP3_ERR_STATE, "loglik_io_bytes: the body is not set");
    // the graph's parameter copy (cp3_loglik_evaluate fills kOscBlock and one
    // rho*Ye per layer) and the rows the layer kernel writes
    if (host_to_device) *host_to_device = (long long)(kOscBlock + sizeof(double) * (L->n_rows + 1));
    if (device_to_host) *device_to_host = (long long)sizeof(double) * L->n_en * (7 + L->n_rows);
    return CP3_OK;
}

}  // extern "C"

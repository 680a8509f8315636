// Kernels of the single-grid propagator:
//   prep_kernel       FP64 per-(energy, layer) eigen data and per-(cosine,
//                     layer) segment lengths (replaces the per-pair getMfast /
//                     get_product work of physics.hpp:268-431, which depends on
//                     energy and layer only);
//   propagate_kernel  one thread per (cosine, energy) pair: layer chain and
//                     probability writeback (physics.hpp:583-702).
//
// Data layout in HBM (n_en_pad = energies rounded up to the tile TE):
//   tab   tile-major [n_en_pad/TE][nl][W][TE] words, W = 13 (mixed: 9 Q1.30
//         overlap entries T_l then kappa1 hi/lo, kappa2 hi/lo as float bits)
//         or 11 doubles (FP64: T_l, kappa1, kappa2); one block stages its
//         energy tile with one contiguous copy.
//   pe    [18][n_en_pad] Lambda' (rows e, mu of W V_1) and Gamma' (columns e, mu of
//         V_0^T W^dagger), Q1.30 or double
//   len   [n_cos][nl_pad] segment lengths in km (float2 hi/lo or double)
//   out   [9][n_cos][n_en] probabilities, plane in*3+out (physics.hpp:689-691)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "cp3_chain.cuh"
#include "cp3_launch.h"
#include "cp3_physics.cuh"

namespace cp3 {

// ------------------------------------------------------------------ prep ----
// Energy part: a block of (nl x eb) threads; thread (l, e) solves layer l at
// energy e, the eigenvectors go through shared memory so that the same thread
// can form the overlap T_l = V_{l+1}^T V_l.  Cosine part: one thread per
// cosine, all segment lengths of that trajectory.
template <bool MIXED>
__global__ void __launch_bounds__(256) prep_kernel(PrepArgs a) {
    extern __shared__ double s_v[];  // [eb][nl][9]
    const int nl = a.pb.nl;
    const int eb = blockDim.y;
    if ((int)blockIdx.x < a.n_energy_blocks) {
        const int l = threadIdx.x, ey = threadIdx.y;
        const int e = blockIdx.x * eb + ey;
        const bool live = (l < nl) && (e < a.pb.n_en_pad);
        const int te = a.pb.te, tile = e / te, lane = e % te;
        const int W = MIXED ? kMixedWords : kFp64Words;
        double* vme = s_v + ((size_t)ey * nl + (l < nl ? l : 0)) * 9;
        if (live) {
            const double E = a.pb.energies[e < a.pb.n_en ? e : a.pb.n_en - 1];
            double m[3], V[9];
            layer_eigen(a.osc, E, a.pb.rhoye[l], m, V);
            for (int w = 0; w < 9; w++) vme[w] = V[w];
            const double k1 = phase_turns_per_km(m[1], m[0], E);
            const double k2 = phase_turns_per_km(m[2], m[0], E);
            const size_t base = ((size_t)tile * nl + l) * W * te + lane;
            if (MIXED) {
                int* t = (int*)a.tab;
                const float k1h = (float)k1, k2h = (float)k2;
                t[base + 9 * (size_t)te] = __float_as_int(k1h);
                t[base + 10 * (size_t)te] = __float_as_int((float)(k1 - (double)k1h));
                t[base + 11 * (size_t)te] = __float_as_int(k2h);
                t[base + 12 * (size_t)te] = __float_as_int((float)(k2 - (double)k2h));
            } else {
                double* t = (double*)a.tab;
                t[base + 9 * (size_t)te] = k1;
                t[base + 10 * (size_t)te] = k2;
            }
            if (l <= 1) {
                // per energy: Gamma' = columns e, mu of V_0^T W^dagger (l = 0) and
                // Lambda' = rows e, mu of W V_1 (l = 1), W = R23 diag(1, 1, e^{i dcp})
                const double c23 = a.osc.c23, s23 = a.osc.s23, cd = a.osc.cd, sd = a.osc.sd;
                const double sg = (l == 0) ? -1.0 : 1.0;  // e^{-i dcp} for Gamma', e^{+i dcp} for Lambda'
                double w[18];
                for (int k = 0; k < 3; k++) {
                    w[k] = V[k];  // row 0 of V (l = 1) / column 0 of V^T (l = 0): V[0][k]
                    w[3 + 2 * k] = c23 * V[3 + k] + s23 * cd * V[6 + k];
                    w[4 + 2 * k] = sg * s23 * sd * V[6 + k];
                }
                const int off = (l == 0) ? 9 : 0;
                for (int q = 0; q < 9; q++) {
                    const size_t idx = (size_t)(off + q) * a.pb.n_en_pad + e;
                    if (MIXED)
                        ((int*)a.pe)[idx] = __double2int_rn(w[q] * 1073741824.0);
                    else
                        ((double*)a.pe)[idx] = w[q];
                }
            }
        }
        __syncthreads();
        if (live) {
            // T_l = V_{l+1}^T V_l; the innermost layer has no successor and
            // keeps the identity so that the table is defined everywhere
            const size_t base = ((size_t)tile * nl + l) * W * te + lane;
            const double* vn = vme + 9;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const double tij = (l + 1 < nl)
                        ? vn[i] * vme[j] + vn[3 + i] * vme[3 + j] + vn[6 + i] * vme[6 + j]
                        : (i == j ? 1.0 : 0.0);
                    if (MIXED)
                        ((int*)a.tab)[base + (size_t)(3 * i + j) * te] = __double2int_rn(tij * 1073741824.0);
                    else
                        ((double*)a.tab)[base + (size_t)(3 * i + j) * te] = tij;
                }
        }
    } else {
        const int c = (blockIdx.x - a.n_energy_blocks) * (blockDim.x * blockDim.y) +
                      threadIdx.y * blockDim.x + threadIdx.x;
        if (c >= a.pb.n_cos) return;
        const double cz = a.pb.cosines[c];
        const int M = a.pb.maxlayers[c];
        const double path = path_length_cm(cz, a.pb.height_cm);
        for (int l = 0; l < a.pb.nl_pad; l++) {
            const double L = (l <= M) ? layer_length_km(a.pb.radii, l, M, cz, path) : 0.0;
            const size_t idx = (size_t)c * a.pb.nl_pad + l;
            if (MIXED) {
                const float h = (float)L;
                ((float2*)a.len)[idx] = make_float2(h, (float)(L - (double)h));
            } else {
                ((double*)a.len)[idx] = L;
            }
        }
    }
}

// ------------------------------------------------------------ propagate ----
template <int TE>
struct MixedSrc {
    const int* tab;    // shared: [nl][13][TE], offset by the thread's lane
    const int* pe;     // shared: [18][TE], offset by lane
    const float2* len; // shared: this cosine's [nl_pad]
    const int4* ptab;  // shared: 257 (Q1.30 cos, sin, float cos, sin)
    __device__ __forceinline__ int T(int l, int i, int j) const { return tab[(l * kMixedWords + 3 * i + j) * TE]; }
    __device__ __forceinline__ int La(int j) const { return pe[j * TE]; }
    __device__ __forceinline__ Q30::C Lb(int j) const { return Q30::C{pe[(3 + 2 * j) * TE], pe[(4 + 2 * j) * TE]}; }
    __device__ __forceinline__ int Ga(int k) const { return pe[(9 + k) * TE]; }
    __device__ __forceinline__ Q30::C Gb(int k) const { return Q30::C{pe[(12 + 2 * k) * TE], pe[(13 + 2 * k) * TE]}; }
    __device__ __forceinline__ void phase(int l, int& c1, int& s1, int& n1, int& c2, int& s2, int& n2) const {
        const float2 L = len[l];
        const int* k = tab + (l * kMixedWords + 9) * TE;
        phase_q30(__int_as_float(k[0]), __int_as_float(k[TE]), L.x, L.y, ptab, c1, s1);
        phase_q30(__int_as_float(k[2 * TE]), __int_as_float(k[3 * TE]), L.x, L.y, ptab, c2, s2);
        n1 = -s1;
        n2 = -s2;
    }
};

template <int TE>
struct F64Src {
    const double* tab;  // shared: [nl][11][TE], offset by lane
    const double* pe;
    const double* len;
    __device__ __forceinline__ double T(int l, int i, int j) const { return tab[(l * kFp64Words + 3 * i + j) * TE]; }
    __device__ __forceinline__ double La(int j) const { return pe[j * TE]; }
    __device__ __forceinline__ F64::C Lb(int j) const { return F64::C{pe[(3 + 2 * j) * TE], pe[(4 + 2 * j) * TE]}; }
    __device__ __forceinline__ double Ga(int k) const { return pe[(9 + k) * TE]; }
    __device__ __forceinline__ F64::C Gb(int k) const { return F64::C{pe[(12 + 2 * k) * TE], pe[(13 + 2 * k) * TE]}; }
    __device__ __forceinline__ void phase(int l, double& c1, double& s1, double& n1, double& c2, double& s2,
                                          double& n2) const {
        const double L = len[l];
        const double* k = tab + (l * kFp64Words + 9) * TE;
        phase_f64(k[0], L, c1, s1);
        phase_f64(k[TE], L, c2, s2);
        n1 = -s1;
        n2 = -s2;
    }
};

// Copy `n16` 16-byte units from global to shared with the whole block.
__device__ __forceinline__ void block_copy16(void* dst, const void* src, int n16) {
    const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
    int4* d = (int4*)dst;
    const int4* s = (const int4*)src;
    for (int i = t; i < n16; i += nt) d[i] = __ldg(s + i);
}

template <bool MIXED, int TE>
__global__ void __launch_bounds__(MIXED ? 256 : 128, 3) propagate_kernel(PropArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    using Word = typename std::conditional<MIXED, int, double>::type;
    constexpr int W = MIXED ? kMixedWords : kFp64Words;
    const int tile = blockIdx.x;
    const int c0 = blockIdx.y * a.cchunk;
    const int c1 = min(c0 + a.cchunk, a.n_cos);
    const int ncl = c1 - c0;

    // stage: energy-tile table, V_0/V_1, phase table, lengths and layer counts
    Word* s_tab = (Word*)smem;
    const size_t tab_words = (size_t)a.nl * W * TE;
    Word* s_pe = s_tab + tab_words;
    int4* s_ptab = (int4*)(s_pe + kPerEWords * TE);
    unsigned char* after_ptab = (unsigned char*)s_ptab + (MIXED ? kPhaseTabBytes : 0);
    unsigned char* s_len_raw = after_ptab;
    int* s_maxl = (int*)(s_len_raw + (size_t)a.cchunk * a.nl_pad * 8);

    block_copy16(s_tab, (const Word*)a.tab + (size_t)tile * tab_words, (int)(tab_words * sizeof(Word) / 16));
    {
        const int nt = blockDim.x * blockDim.y, t = threadIdx.y * blockDim.x + threadIdx.x;
        const Word* pe = (const Word*)a.pe;
        for (int i = t; i < kPerEWords * TE; i += nt) {
            const int w = i / TE, lane = i % TE;
            s_pe[i] = pe[(size_t)w * a.n_en_pad + (size_t)tile * TE + lane];
        }
        if (MIXED)
            for (int i = t; i < kPhaseTabN + 1; i += nt) s_ptab[i] = a.ptab[i];
        const int nlen16 = ncl * a.nl_pad / 2;  // 8-byte entries, nl_pad even
        block_copy16(s_len_raw, (const unsigned char*)a.len + (size_t)c0 * a.nl_pad * 8, nlen16);
        for (int i = t; i < ncl; i += nt) s_maxl[i] = a.maxl[c0 + i];
    }
    __syncthreads();

    const int lane = threadIdx.x;
    const int e = tile * TE + lane;
    const bool store = e < a.n_en;
    const size_t plane = (size_t)a.n_cos * a.n_en;
    for (int cl = threadIdx.y; cl < ncl; cl += blockDim.y) {
        const int M = s_maxl[cl];
        const int ci = c0 + cl;
        if (MIXED) {
            MixedSrc<TE> src{(const int*)s_tab + lane, (const int*)s_pe + lane,
                             (const float2*)s_len_raw + (size_t)cl * a.nl_pad, s_ptab};
            const Q30 ar{a.bias};
            Q30::C B[4];
            flavour_block<Q30>(ar, src, M, B);
            float pr[9];
            Q30::complete(B, pr);
            if (store) {
                float* out = (float*)a.out + (size_t)ci * a.n_en + e;
#pragma unroll
                for (int t = 0; t < 9; t++) __stcs(out + (size_t)t * plane, pr[t]);
            }
        } else {
            F64Src<TE> src{(const double*)s_tab + lane, (const double*)s_pe + lane,
                           (const double*)s_len_raw + (size_t)cl * a.nl_pad};
            const F64 ar{};
            F64::C B[4];
            flavour_block<F64>(ar, src, M, B);
            double pr[9];
            F64::complete(B, pr);
            if (store) {
                double* out = (double*)a.out + (size_t)ci * a.n_en + e;
#pragma unroll
                for (int t = 0; t < 9; t++) __stcs(out + (size_t)t * plane, pr[t]);
            }
        }
    }
}

// ------------------------------------------------------------- launchers ----
size_t propagate_smem_bytes(bool mixed, int te, int nl, int nl_pad, int cchunk) {
    const size_t word = mixed ? 4 : 8;
    const size_t W = mixed ? kMixedWords : kFp64Words;
    size_t b = (size_t)nl * W * te * word + (size_t)kPerEWords * te * word;
    if (mixed) b += kPhaseTabBytes;
    b += (size_t)cchunk * nl_pad * 8 + (size_t)cchunk * 4;
    return (b + 15) / 16 * 16;
}

cudaError_t launch_prep(bool mixed, PrepArgs a, cudaStream_t s) {
    // energy blocks: (nl x eb) threads with eb = max(1, 256 / nl)
    const int nl = a.pb.nl;
    const int eb = std::max(1, 256 / nl);
    a.n_energy_blocks = (a.pb.n_en_pad + eb - 1) / eb;
    const int threads = nl * eb;
    const int nbC = (a.pb.n_cos + threads - 1) / threads;
    const size_t smem = (size_t)eb * nl * 9 * sizeof(double);
    if (a.n_energy_blocks + nbC == 0) return cudaSuccess;
    dim3 block(nl, eb);
    if (mixed)
        prep_kernel<true><<<a.n_energy_blocks + nbC, block, smem, s>>>(a);
    else
        prep_kernel<false><<<a.n_energy_blocks + nbC, block, smem, s>>>(a);
    return cudaGetLastError();
}

template <bool MIXED, int TE>
static cudaError_t launch_prop_t(const PropArgs& a, int groups, size_t smem, cudaStream_t s) {
    static bool configured = false;  // one attribute call per instantiation (per process)
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(propagate_kernel<MIXED, TE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid(a.n_en_pad / TE, (a.n_cos + a.cchunk - 1) / a.cchunk);
    dim3 block(TE, groups);
    propagate_kernel<MIXED, TE><<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_propagate(bool mixed, const PropArgs& a, int te, int groups, size_t smem, cudaStream_t s) {
    if (a.n_cos == 0 || a.n_en == 0) return cudaSuccess;
    if (mixed) {
        if (te == 32) return launch_prop_t<true, 32>(a, groups, smem, s);
        if (te == 64) return launch_prop_t<true, 64>(a, groups, smem, s);
        if (te == 128) return launch_prop_t<true, 128>(a, groups, smem, s);
    } else {
        if (te == 32) return launch_prop_t<false, 32>(a, groups, smem, s);
        if (te == 64) return launch_prop_t<false, 64>(a, groups, smem, s);
        if (te == 128) return launch_prop_t<false, 128>(a, groups, smem, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cp3

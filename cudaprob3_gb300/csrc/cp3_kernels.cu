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
#include <mutex>
#include <set>
#include <type_traits>
#include <utility>

#include "cp3_launch.h"
#include "cp3_tile.cuh"

namespace cp3 {

// ------------------------------------------------------------------ prep ----
// Energy part: a block of (nl x eb) threads; thread (l, e) solves layer l at
// energy e, the eigenvectors go through shared memory so that the same thread
// can form the overlap T_l = V_{l+1}^T V_l.  Cosine part: one thread per
// (cosine, layer) segment length, and the atmosphere segments of the
// production heights spread over the cosine's layer threads.
template <bool MIXED>
__global__ void __launch_bounds__(256) prep_kernel(PrepArgs a) {
    extern __shared__ double s_v[];  // [eb][nl][9]
    const int nl = a.pb.nl;
    const int eb = blockDim.y;
    const GridTables g{a.tab, a.pe, a.len, a.pb.n_en_pad, a.pb.te, nl, a.pb.nl_pad};
    if ((int)blockIdx.x < a.n_energy_blocks) {
        const int l = threadIdx.x, ey = threadIdx.y;
        const int e = blockIdx.x * eb + ey;
        const bool live = (l < nl) && (e < a.pb.n_en_pad);
        double* vme = s_v + ((size_t)ey * nl + (l < nl ? l : 0)) * 9;
        if (live) {
            const double E = a.pb.energies[e < a.pb.n_en ? e : a.pb.n_en - 1];
            prep_energy_layer<MIXED>(a.osc, E, a.pb.rhoye[l], l, e, g, vme);
        }
        __syncthreads();
        if (live) prep_overlap<MIXED>(l, e, g, vme);
    } else {
        // one thread per (cosine, layer)
        const long long f = (long long)(blockIdx.x - a.n_energy_blocks) * (blockDim.x * blockDim.y) +
                            threadIdx.y * blockDim.x + threadIdx.x;
        const int c = (int)(f / a.pb.nl_pad), l = (int)(f % a.pb.nl_pad);
        if (c >= a.pb.n_cos) return;
        const double cz = a.pb.cosines[c];
        const int M = a.pb.maxlayers[c];
        if (!check_ok(kSitePrepLayer, M, nl)) return;
        prep_cosine_layer<MIXED>(cz, M, a.pb.radii, a.pb.height_cm, c, l, g);
        // atmosphere segment at every production height (physics.hpp:613-616,
        // 561-562), spread over the cosine's layer threads
        for (int h = l; h < a.n_h; h += a.pb.nl_pad) {
            const double L0 = layer_length_km(a.pb.radii, 0, M, cz, path_length_cm(cz, a.heights_cm[h]));
            const size_t idx = (size_t)c * a.n_h + h;
            if (MIXED) {
                const float hi = f32_rn(L0);
                ((float2*)a.lenh)[idx] = make_float2(hi, f32_rn(L0 - f64_of(hi)));
            } else {
                ((double*)a.lenh)[idx] = L0;
            }
        }
    }
}

// ------------------------------------------------------------ propagate ----
// Mixed: 4 blocks of 256 threads per SM (64 registers; planes and height
// averages without spill: the atmosphere segment is formed after the layer
// chain; the height-average mode ran 1.2 % faster at 4 blocks than at 3);
// FP64: registers for 3 blocks of 128 threads, of which its shared memory
// (the double tables, about 90 KB at 13 layers) leaves 2 per SM -- 8 warps,
// enough for the FP64 pipe, which it keeps over 90 % busy.
template <bool MIXED, int TE, int MODE>
__global__ void __launch_bounds__(MIXED ? 256 : 128, MIXED ? 4 : 3)
    propagate_kernel(PropArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const TileSmem L = tile_smem(MIXED, TE, a.nl, a.nl_pad, a.cchunk);
    stage_phase_table<MIXED>(smem, L, a.ptab);
    TileJob j;
    j.tab = a.tab;
    j.pe = a.pe;
    j.len = a.len;
    j.maxl = a.maxl;
    j.out = a.out;
    j.n_cos = a.n_cos;
    j.n_en = a.n_en;
    j.n_en_pad = a.n_en_pad;
    j.etile = blockIdx.x;
    j.c0 = blockIdx.y * a.cchunk;
    j.ncl = min(j.c0 + a.cchunk, a.n_cos) - j.c0;
    j.flux = a.flux;
    j.flux_mask = a.flux_mask;
    j.cbin = a.cbin;
    j.ebin = a.ebin;
    j.hist = a.hist;
    j.n_cb = a.n_cb;
    j.n_eb = a.n_eb;
    j.lenh = a.lenh;
    j.hw = a.hw;
    j.n_h = a.n_h;
    process_tile<MIXED, TE, MODE>(j, a.nl, a.nl_pad, smem, L);
}

// ------------------------------------------------------------- launchers ----
cudaError_t kernels_check_take(CheckRecord* out) { return check_take(out); }

int max_dynamic_smem() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return 227 * 1024;
    }
    return v;
}

size_t propagate_smem_bytes(bool mixed, int te, int nl, int nl_pad, int cchunk) {
    return tile_smem(mixed, te, nl, nl_pad, cchunk).total;
}

cudaError_t launch_prep(bool mixed, PrepArgs a, cudaStream_t s) {
    // energy blocks: (nl x eb) threads with eb = max(1, 256 / nl)
    const int nl = a.pb.nl;
    const int eb = std::max(1, 256 / nl);
    a.n_energy_blocks = (a.pb.n_en_pad + eb - 1) / eb;
    const int threads = nl * eb;
    const long long nbC = ((long long)a.pb.n_cos * a.pb.nl_pad + threads - 1) / threads;
    const size_t smem = (size_t)eb * nl * 9 * sizeof(double);
    if (a.n_energy_blocks + nbC == 0) return cudaSuccess;
    dim3 block(nl, eb);
    if (mixed)
        prep_kernel<true><<<a.n_energy_blocks + nbC, block, smem, s>>>(a);
    else
        prep_kernel<false><<<a.n_energy_blocks + nbC, block, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t opt_in_max_smem(const void* func) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;  // (kernel, device) pairs already opted in
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({func, dev})) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem());
    if (e == cudaSuccess) done.insert({func, dev});
    return e;
}

template <bool MIXED, int TE, int MODE>
static cudaError_t launch_prop_t(const PropArgs& a, int groups, size_t smem, cudaStream_t s) {
    cudaError_t e = opt_in_max_smem((const void*)propagate_kernel<MIXED, TE, MODE>);
    if (e != cudaSuccess) return e;
    dim3 grid(a.n_en_pad / TE, (a.n_cos + a.cchunk - 1) / a.cchunk);
    dim3 block(TE, groups);
    propagate_kernel<MIXED, TE, MODE><<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_prop_r(bool mixed, const PropArgs& a, int te, int groups, size_t smem, cudaStream_t s) {
    if (mixed) {
        if (te == 32) return launch_prop_t<true, 32, MODE>(a, groups, smem, s);
        if (te == 64) return launch_prop_t<true, 64, MODE>(a, groups, smem, s);
        if (te == 128) return launch_prop_t<true, 128, MODE>(a, groups, smem, s);
    } else {
        if (te == 32) return launch_prop_t<false, 32, MODE>(a, groups, smem, s);
        if (te == 64) return launch_prop_t<false, 64, MODE>(a, groups, smem, s);
        if (te == 128) return launch_prop_t<false, 128, MODE>(a, groups, smem, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_propagate(bool mixed, const PropArgs& a, int te, int groups, size_t smem, cudaStream_t s,
                             int mode) {
    if (a.n_cos == 0 || a.n_en == 0) return cudaSuccess;
    if (mode == kModeRates) return launch_prop_r<kModeRates>(mixed, a, te, groups, smem, s);
    if (mode == kModeHeights) return launch_prop_r<kModeHeights>(mixed, a, te, groups, smem, s);
    if (mode == kModeBlock) return launch_prop_r<kModeBlock>(mixed, a, te, groups, smem, s);
    return launch_prop_r<kModePlanes>(mixed, a, te, groups, smem, s);
}

}  // namespace cp3

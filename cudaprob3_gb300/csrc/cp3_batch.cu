// Batched propagation: many independent parameter sets, each with its own
// oscillation parameters, density scale and (cosine x energy) grid, evaluated
// by one persistent kernel launch inside a CUDA graph.
//
// No reference counterpart: CUDAProb3++ evaluates one parameter point per
// calculateProbabilities call (cudapropagator.cuh:162-220).  Each set here is
// exactly that computation, with the results of set s in the reference's
// layout [9][n_cos_s][n_en_s] at element offset out_offset[s].
//
// Device work:
//   batch_prep_kernel       eigen data of every (set, energy, layer) (double-float
//                           solve for the mixed tables, FP64 for the FP64 ones)
//                           and segment lengths of every (set, cosine, layer)
//   batch_propagate_kernel  persistent: each block takes (set, energy tile,
//                           cosine chunk) items from an atomic counter, largest
//                           items first, and runs process_tile on them
// The sets are split into up to 8 chunks of geometrically growing work; the
// graph is a counter reset, then per chunk a prep launch on a low-priority
// side stream and the chunk's persistent propagate launch on the
// high-priority main stream, so that chunk k + 1's prep runs beside chunk k's
// propagation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "cudaprob3_gb300.h"
#include "cp3_launch.h"
#include "cp3_tile.cuh"

namespace cp3 {

struct BatchGrid {
    OscParams osc;
    int n_cos, n_en, n_en_pad;
    long long cos_off, en_off;          // into the concatenated cosines/energies/maxlayers
    long long tab_off, pe_off, len_off;  // words (tab, pe) and 8-byte entries (len)
    long long out_off;                   // elements
    int rhoye_off;                       // into rhoye [n_sets][nl]
};

struct BatchPrepArgs {
    const BatchGrid* grids;
    const int2* eblk;  // (set, first energy) of each energy block
    const int2* cblk;  // (set, first cosine) of each cosine block
    int n_eblk, n_cblk, eb;
    const double* energies;
    const double* cosines;
    const int* maxl;
    const double* radii;
    const double* rhoye;
    double height_cm;
    int nl, nl_pad, te;
    void* tab;
    void* pe;
    void* len;
    // extents for the checked build: sets, table words, length entries
    int n_sets;
    long long tab_words, pe_words, len_entries;
};

// Checked build: the tables of set `gr` lie inside the batch's buffers.
__device__ __forceinline__ bool batch_grid_ok(const BatchGrid& gr, int nl, int nl_pad, int W, long long tab_words,
                                              long long pe_words, long long len_entries) {
    return check_ok(kSiteBatchTile, gr.tab_off + (long long)gr.n_en_pad * nl * W - 1, tab_words) &&
           check_ok(kSiteBatchTile, gr.pe_off + (long long)kPerEWords * gr.n_en_pad - 1, pe_words) &&
           (gr.n_cos == 0 || check_ok(kSiteBatchTile, gr.len_off + (long long)gr.n_cos * nl_pad - 1, len_entries));
}

template <bool MIXED>
__device__ __forceinline__ void batch_prep_item(const BatchPrepArgs& a, int bid) {
    extern __shared__ double s_v[];
    const int nl = a.nl;
    // cosine blocks first: blocks dispatch in index order, and the short
    // cosine blocks would otherwise trail the eigen-solves
    const int W = MIXED ? kMixedWords : kFp64Words;
    if ((int)bid >= a.n_cblk) {
        const int2 b = a.eblk[bid - a.n_cblk];
        if (!check_ok(kSiteBatchSet, b.x, a.n_sets)) return;  // b is the same for the whole block
        const BatchGrid& gr = a.grids[b.x];
        if (!(batch_grid_ok(gr, nl, a.nl_pad, W, a.tab_words, a.pe_words, a.len_entries) &&
              check_ok(kSiteBatchPrep, b.y, gr.n_en_pad)))
            return;
        const size_t word = MIXED ? 4 : 8;
        const GridTables g{(unsigned char*)a.tab + gr.tab_off * word, (unsigned char*)a.pe + gr.pe_off * word,
                           (unsigned char*)a.len + gr.len_off * 8, gr.n_en_pad, a.te, nl, a.nl_pad};
        const int l = threadIdx.x, ey = threadIdx.y;
        const int e = b.y + ey;
        const bool live = (l < nl) && (e < gr.n_en_pad);
        const int nt = nl * blockDim.y;
        if (nt <= 32) {
            // one warp: the next layer's eigenvectors come from the next lane,
            // and the block needs no shared memory (so that it fits beside the
            // persistent propagate blocks, which take nearly all of it)
            double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vn[9];
            if (live) {
                const double E = a.energies[gr.en_off + (e < gr.n_en ? e : gr.n_en - 1)];
                prep_energy_layer<MIXED>(gr.osc, E, a.rhoye[gr.rhoye_off + l], l, e, g, v);
            }
            const unsigned mask = (nt == 32) ? 0xffffffffu : ((1u << nt) - 1u);
#pragma unroll
            for (int q = 0; q < 9; q++) vn[q] = __shfl_down_sync(mask, v[q], 1);
            if (live) prep_overlap_v<MIXED>(l, e, g, v, vn);
        } else {
            double* vme = s_v + ((size_t)ey * nl + (l < nl ? l : 0)) * 9;
            if (live) {
                const double E = a.energies[gr.en_off + (e < gr.n_en ? e : gr.n_en - 1)];
                prep_energy_layer<MIXED>(gr.osc, E, a.rhoye[gr.rhoye_off + l], l, e, g, vme);
            }
            __syncthreads();
            if (live) prep_overlap<MIXED>(l, e, g, vme);
        }
    } else {
        const int2 b = a.cblk[bid];
        if (!check_ok(kSiteBatchSet, b.x, a.n_sets)) return;
        const BatchGrid& gr = a.grids[b.x];
        if (!batch_grid_ok(gr, nl, a.nl_pad, W, a.tab_words, a.pe_words, a.len_entries)) return;
        // one thread per (cosine, layer): b.y is the block's first flat index
        const int f = b.y + threadIdx.y * blockDim.x + threadIdx.x;
        const int c = f / a.nl_pad, l = f % a.nl_pad;
        if (c >= gr.n_cos) return;
        const size_t word = MIXED ? 4 : 8;
        const GridTables g{(unsigned char*)a.tab + gr.tab_off * word, (unsigned char*)a.pe + gr.pe_off * word,
                           (unsigned char*)a.len + gr.len_off * 8, gr.n_en_pad, a.te, nl, a.nl_pad};
        prep_cosine_layer<MIXED>(a.cosines[gr.cos_off + c], a.maxl[gr.cos_off + c], a.radii, a.height_cm, c, l, g);
    }
}

// A grid of at most a few blocks per SM loops over the prep items: the items
// run beside the persistent propagate wave of the previous chunk, and fewer,
// longer-lived blocks keep the block scheduler out of its way.
template <bool MIXED>
__global__ void __launch_bounds__(256) batch_prep_kernel(BatchPrepArgs a) {
    const int n = a.n_eblk + a.n_cblk;
    for (int bid = blockIdx.x; bid < n; bid += gridDim.x) batch_prep_item<MIXED>(a, bid);
}

struct BatchPropArgs {
    const BatchGrid* grids;
    const int4* items;  // (set, energy tile, first cosine, cosines)
    int n_items;
    int* counter;
    const void* tab;
    const void* pe;
    const void* len;
    const int* maxl;
    const int4* ptab;
    void* out;
    int nl, nl_pad, cchunk;
    // extents for the checked build
    int n_sets;
    long long tab_words, pe_words, len_entries, out_elems;
};

template <bool MIXED, int TE>
__global__ void __launch_bounds__(MIXED ? 256 : 128, MIXED ? 4 : 3) batch_propagate_kernel(BatchPropArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const TileSmem L = tile_smem(MIXED, TE, a.nl, a.nl_pad, a.cchunk);
    int& s_item = *(int*)(smem + L.total);  // work-item slot after the tile (all shared memory is dynamic)
    stage_phase_table<MIXED>(smem, L, a.ptab);
    const size_t word = MIXED ? 4 : 8;
    const size_t osz = MIXED ? sizeof(float) : sizeof(double);
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const int4 w = a.items[it];
        // checked build: the item names a set whose tables and planes lie in
        // the batch's buffers (w is the same for the whole block)
        const bool item_ok = check_ok(kSiteBatchSet, w.x, a.n_sets);
        const BatchGrid& g = a.grids[item_ok ? w.x : 0];
        TileJob j;
        j.tab = (const unsigned char*)a.tab + g.tab_off * word;
        j.pe = (const unsigned char*)a.pe + g.pe_off * word;
        j.len = (const unsigned char*)a.len + g.len_off * 8;
        j.maxl = a.maxl + g.cos_off;
        j.out = (unsigned char*)a.out + g.out_off * osz;
        j.n_cos = g.n_cos;
        j.n_en = g.n_en;
        j.n_en_pad = g.n_en_pad;
        j.etile = w.y;
        j.c0 = w.z;
        j.ncl = w.w;
        if (item_ok && batch_grid_ok(g, a.nl, a.nl_pad, MIXED ? kMixedWords : kFp64Words, a.tab_words, a.pe_words,
                                     a.len_entries) &&
            ((long long)g.n_cos * g.n_en == 0 ||
             check_ok(kSiteBatchTile, g.out_off + 9LL * g.n_cos * g.n_en - 1, a.out_elems)))
            process_tile<MIXED, TE>(j, a.nl, a.nl_pad, smem, L);
        __syncthreads();
    }
}

template <bool MIXED, int TE>
static cudaError_t batch_attr() {
    return opt_in_max_smem((const void*)batch_propagate_kernel<MIXED, TE>);
}

template <bool MIXED, int TE>
static cudaError_t batch_launch_t(const BatchPropArgs& a, int groups, size_t smem, int blocks, cudaStream_t s) {
    cudaError_t e = batch_attr<MIXED, TE>();
    if (e != cudaSuccess) return e;
    batch_propagate_kernel<MIXED, TE><<<blocks, dim3(TE, groups), smem, s>>>(a);
    return cudaGetLastError();
}

template <bool MIXED, int TE>
static cudaError_t batch_occupancy_t(int groups, size_t smem, int* blocks_per_sm) {
    cudaError_t e = batch_attr<MIXED, TE>();
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_propagate_kernel<MIXED, TE>,
                                                         TE * groups, smem);
}

static cudaError_t batch_launch(bool mixed, int te, const BatchPropArgs& a, int groups, size_t smem, int blocks,
                                cudaStream_t s) {
    if (mixed) {
        if (te == 32) return batch_launch_t<true, 32>(a, groups, smem, blocks, s);
        if (te == 64) return batch_launch_t<true, 64>(a, groups, smem, blocks, s);
        if (te == 128) return batch_launch_t<true, 128>(a, groups, smem, blocks, s);
    } else {
        if (te == 32) return batch_launch_t<false, 32>(a, groups, smem, blocks, s);
        if (te == 64) return batch_launch_t<false, 64>(a, groups, smem, blocks, s);
        if (te == 128) return batch_launch_t<false, 128>(a, groups, smem, blocks, s);
    }
    return cudaErrorInvalidValue;
}

static cudaError_t batch_occupancy(bool mixed, int te, int groups, size_t smem, int* bps) {
    if (mixed) {
        if (te == 32) return batch_occupancy_t<true, 32>(groups, smem, bps);
        if (te == 64) return batch_occupancy_t<true, 64>(groups, smem, bps);
        if (te == 128) return batch_occupancy_t<true, 128>(groups, smem, bps);
    } else {
        if (te == 32) return batch_occupancy_t<false, 32>(groups, smem, bps);
        if (te == 64) return batch_occupancy_t<false, 64>(groups, smem, bps);
        if (te == 128) return batch_occupancy_t<false, 128>(groups, smem, bps);
    }
    return cudaErrorInvalidValue;
}

static cudaError_t batch_prep_launch(bool mixed, const BatchPrepArgs& a, cudaStream_t s, int max_blocks) {
    const int blocks = std::min(a.n_eblk + a.n_cblk, std::max(1, max_blocks));
    if (a.n_eblk + a.n_cblk == 0) return cudaSuccess;
    dim3 block(a.nl, a.eb);
    const size_t smem = (a.nl * a.eb <= 32) ? 0 : (size_t)a.eb * a.nl * 9 * sizeof(double);
    if (mixed)
        batch_prep_kernel<true><<<blocks, block, smem, s>>>(a);
    else
        batch_prep_kernel<false><<<blocks, block, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace cp3

// ======================================================================= host
namespace {

int bfail(int code, const std::string& m) {
    cp3::set_last_error(m);
    return code;
}
int bcuda(cudaError_t e, const char* where) {
    return bfail(CP3_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

struct Guard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit Guard(int d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) err = cudaSetDevice(d);
    }
    ~Guard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (p && count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct cp3_batch {
    int device = 0;
    bool mixed = true;
    int n_sets = 0;
    std::vector<int> n_cos, n_en;
    std::vector<long long> cos_off, en_off, out_off;
    long long total_cos = 0, total_en = 0, total_out = 0;

    std::vector<double> cosines, energies;
    std::vector<int> maxl;
    std::vector<double> params;  // [n_sets][6]
    std::vector<double> scale;   // [n_sets]
    std::vector<double> radii, rhos, ye, coslimit;
    double height_cm = 0;
    bool has_grids = false, has_params = false, has_density = false, has_height = false;
    int type = -1;

    int te = 64, groups = 4, cchunk = 32;
    bool layout_dirty = true, inputs_dirty = true, desc_dirty = true;

    cudaStream_t own = nullptr, stream = nullptr;
    DBuf<double> d_cos, d_en, d_radii, d_rhoye;
    DBuf<int> d_maxl, d_counter;
    DBuf<cp3::BatchGrid> d_grids;
    DBuf<int2> d_eblk, d_cblk;
    DBuf<int4> d_items, d_ptab;
    DBuf<unsigned char> d_tab, d_pe, d_len, d_out;

    std::vector<cp3::BatchGrid> grids;
    std::vector<int2> eblk, cblk;
    std::vector<int4> items;
    // the sets are split into chunks of about equal work: chunk k's prep runs
    // while the persistent kernel propagates chunk k - 1 (offsets into the
    // lists above, n_chunks + 1 entries each)
    int n_chunks = 0;
    std::vector<int> chunk_eblk, chunk_cblk, chunk_items;
    int nl = 0, nl_pad = 0, eb = 1, blocks = 0;
    size_t smem = 0;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    float last_ms = 0.f;

    size_t elem() const { return mixed ? 4 : 8; }
};

namespace {

void drop_graph(cp3_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

void compute_maxl(cp3_batch* b) {
    for (long long i = 0; i < b->total_cos; i++) {
        int cnt = 0;
        for (double lim : b->coslimit) cnt += (b->cosines[i] < lim);
        b->maxl[i] = cnt;
    }
}

// Host descriptors, block lists and work items for the current launch shape.
int build_layout(cp3_batch* b) {
    const int n = (int)b->radii.size();
    b->nl = n + 1;
    b->nl_pad = (b->nl + 1) / 2 * 2;
    const int W = b->mixed ? cp3::kMixedWords : cp3::kFp64Words;
    // the energy tile must leave room for the layer tables: halve the tile,
    // then the cosine chunk, as the single-grid handle does
    {
        const size_t smem_max = (size_t)cp3::max_dynamic_smem();
        auto need = [&]() { return cp3::tile_smem(b->mixed, b->te, b->nl, b->nl_pad, b->cchunk).total + 16; };
        while (need() > smem_max && b->te > 32) {
            b->te /= 2;
            b->groups = std::min(b->groups * 2, cp3::propagate_max_threads(b->mixed) / b->te);
        }
        while (need() > smem_max && b->cchunk > 8) b->cchunk /= 2;
    }
    // one-warp prep blocks: they run beside the persistent propagate blocks,
    // in the registers and shared memory those leave free
    b->eb = std::max(1, 32 / b->nl);
    b->grids.assign(b->n_sets, cp3::BatchGrid{});
    b->eblk.clear();
    b->cblk.clear();
    b->items.clear();
    b->chunk_eblk.assign(1, 0);
    b->chunk_cblk.assign(1, 0);
    b->chunk_items.assign(1, 0);
    long long tab = 0, pe = 0, len = 0;
    const int cthreads = b->nl * b->eb;
    // work of every set (the chain cost of its cosines times its energy tiles)
    std::vector<double> set_cost(b->n_sets, 0.0);
    double total_cost = 0.0;
    int live_sets = 0;
    for (int s = 0; s < b->n_sets; s++) {
        if (b->n_cos[s] == 0 || b->n_en[s] == 0) continue;
        double c = 0.0;
        for (int i = 0; i < b->n_cos[s]; i++) c += 78.0 * b->maxl[b->cos_off[s] + i] + 116.0;
        set_cost[s] = c * ((b->n_en[s] + b->te - 1) / b->te);
        total_cost += set_cost[s];
        live_sets++;
    }
    const int K = std::max(1, std::min(8, live_sets));
    std::vector<std::pair<double, int4>> work;
    double done = 0.0;
    int chunk = 0;
    // chunk sizes grow geometrically (ratio 1.6): the first chunk's prep is
    // the only one nothing hides, and every later chunk's prep, running in
    // the room the previous chunk's persistent wave leaves, finishes within
    // that chunk's propagation (measured: a prep co-running there proceeds
    // at about twice the work rate of the propagation)
    std::vector<double> bound(K, 1.0);
    {
        double sum = 0.0, w = 1.0;
        for (int k = 0; k < K; k++, w *= 1.6) sum += w;
        double acc = 0.0;
        w = 1.0;
        for (int k = 0; k < K; k++, w *= 1.6) bound[k] = (acc += w / sum);
    }
    auto boundary = [&](int k) { return bound[k]; };
    auto close_chunk = [&]() {
        std::stable_sort(work.begin(), work.end(),
                         [](const std::pair<double, int4>& x, const std::pair<double, int4>& y) { return x.first > y.first; });
        for (auto& w : work) b->items.push_back(w.second);
        work.clear();
        b->chunk_eblk.push_back((int)b->eblk.size());
        b->chunk_cblk.push_back((int)b->cblk.size());
        b->chunk_items.push_back((int)b->items.size());
        chunk++;
    };
    for (int s = 0; s < b->n_sets; s++) {
        cp3::BatchGrid& g = b->grids[s];
        g.n_cos = b->n_cos[s];
        g.n_en = b->n_en[s];
        g.n_en_pad = (g.n_en + b->te - 1) / b->te * b->te;
        g.cos_off = b->cos_off[s];
        g.en_off = b->en_off[s];
        g.out_off = b->out_off[s];
        g.tab_off = tab;
        g.pe_off = pe;
        g.len_off = len;
        g.rhoye_off = s * b->nl;
        tab += (long long)g.n_en_pad * b->nl * W;
        pe += (long long)cp3::kPerEWords * g.n_en_pad;
        len += (long long)g.n_cos * b->nl_pad;
        if (g.n_cos == 0 || g.n_en == 0) continue;
        for (int e0 = 0; e0 < g.n_en_pad; e0 += b->eb) b->eblk.push_back(make_int2(s, e0));
        for (int f0 = 0; f0 < g.n_cos * b->nl_pad; f0 += cthreads) b->cblk.push_back(make_int2(s, f0));
        for (int t = 0; t < g.n_en_pad / b->te; t++)
            for (int c0 = 0; c0 < g.n_cos; c0 += b->cchunk) {
                const int ncl = std::min(b->cchunk, g.n_cos - c0);
                double cost = 0;
                for (int c = c0; c < c0 + ncl; c++) cost += 78.0 * b->maxl[g.cos_off + c] + 116.0;
                work.push_back({cost, make_int4(s, t, c0, ncl)});
            }
        done += set_cost[s];
        if (chunk < K - 1 && done >= total_cost * boundary(chunk)) close_chunk();
    }
    close_chunk();
    b->n_chunks = chunk;
    const size_t word = b->mixed ? 4 : 8;
    cudaError_t e;
    if ((e = b->d_tab.ensure((size_t)tab * word)) != cudaSuccess) return bcuda(e, "cudaMalloc(tables)");
    if ((e = b->d_pe.ensure((size_t)pe * word)) != cudaSuccess) return bcuda(e, "cudaMalloc(tables)");
    if ((e = b->d_len.ensure((size_t)len * 8)) != cudaSuccess) return bcuda(e, "cudaMalloc(lengths)");
    if ((e = b->d_grids.ensure(b->n_sets)) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if ((e = b->d_eblk.ensure(b->eblk.size())) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if ((e = b->d_cblk.ensure(b->cblk.size())) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if ((e = b->d_items.ensure(b->items.size())) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if ((e = b->d_counter.ensure(std::max(1, b->n_chunks))) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if (!b->eblk.empty() &&
        (e = cudaMemcpy(b->d_eblk.p, b->eblk.data(), b->eblk.size() * sizeof(int2), cudaMemcpyHostToDevice)))
        return bcuda(e, "cudaMemcpy");
    if (!b->cblk.empty() &&
        (e = cudaMemcpy(b->d_cblk.p, b->cblk.data(), b->cblk.size() * sizeof(int2), cudaMemcpyHostToDevice)))
        return bcuda(e, "cudaMemcpy");
    if (!b->items.empty() &&
        (e = cudaMemcpy(b->d_items.p, b->items.data(), b->items.size() * sizeof(int4), cudaMemcpyHostToDevice)))
        return bcuda(e, "cudaMemcpy");
    b->smem = cp3::tile_smem(b->mixed, b->te, b->nl, b->nl_pad, b->cchunk).total + 16;  // + work-item slot
    if ((int)b->smem > cp3::max_dynamic_smem())
        return bfail(CP3_ERR_LIMIT, "batch: tile tables exceed shared memory; lower te or cchunk");
    int bps = 0;
    if ((e = cp3::batch_occupancy(b->mixed, b->te, b->groups, b->smem, &bps)) != cudaSuccess)
        return bcuda(e, "occupancy");
    if (bps < 1) return bfail(CP3_ERR_LIMIT, "batch: launch shape does not fit on an SM");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    // one block per SM left free (when 5 or more fit) for the next chunk's
    // prep blocks: the propagation alone measured the same at 5 or 6 blocks
    // per SM, while going from 3 to 2 costs it 4 %
    if (bps >= 5) bps--;
    b->blocks = std::max(1, sms * bps);  // per chunk: at most its item count
    b->layout_dirty = false;
    b->desc_dirty = true;
    drop_graph(b);
    return CP3_OK;
}

// Per-set oscillation parameters (propagator.hpp:191-248) and scaled densities.
int upload_descriptors(cp3_batch* b) {
    std::vector<double> rhoye((size_t)b->n_sets * b->nl);
    for (int s = 0; s < b->n_sets; s++) {
        const double* q = &b->params[6 * s];
        cp3::fill_osc_params(b->grids[s].osc, q[0], q[1], q[2], q[3], q[4], q[5], b->type == CP3_ANTINEUTRINO);
        rhoye[(size_t)s * b->nl] = 0.0;
        for (int i = 0; i < b->nl - 1; i++) rhoye[(size_t)s * b->nl + 1 + i] = b->scale[s] * b->rhos[i] * b->ye[i];
    }
    cudaError_t e;
    if ((e = b->d_rhoye.ensure(rhoye.size())) != cudaSuccess) return bcuda(e, "cudaMalloc");
    if ((e = cudaMemcpyAsync(b->d_rhoye.p, rhoye.data(), rhoye.size() * 8, cudaMemcpyHostToDevice, b->stream)))
        return bcuda(e, "cudaMemcpyAsync");
    if ((e = cudaMemcpyAsync(b->d_grids.p, b->grids.data(), b->grids.size() * sizeof(cp3::BatchGrid),
                             cudaMemcpyHostToDevice, b->stream)))
        return bcuda(e, "cudaMemcpyAsync");
    // the host vectors above must outlive the copies
    if ((e = cudaStreamSynchronize(b->stream))) return bcuda(e, "cudaStreamSynchronize");
    b->desc_dirty = false;
    return CP3_OK;
}

int upload_inputs(cp3_batch* b) {
    cudaError_t e;
    if ((e = b->d_cos.ensure(b->total_cos)) || (e = b->d_en.ensure(b->total_en)) ||
        (e = b->d_maxl.ensure(b->total_cos)) || (e = b->d_radii.ensure(b->radii.size())))
        return bcuda(e, "cudaMalloc");
    if (b->total_cos &&
        ((e = cudaMemcpy(b->d_cos.p, b->cosines.data(), b->total_cos * 8, cudaMemcpyHostToDevice)) ||
         (e = cudaMemcpy(b->d_maxl.p, b->maxl.data(), b->total_cos * 4, cudaMemcpyHostToDevice))))
        return bcuda(e, "cudaMemcpy");
    if (b->total_en && (e = cudaMemcpy(b->d_en.p, b->energies.data(), b->total_en * 8, cudaMemcpyHostToDevice)))
        return bcuda(e, "cudaMemcpy");
    if ((e = cudaMemcpy(b->d_radii.p, b->radii.data(), b->radii.size() * 8, cudaMemcpyHostToDevice)))
        return bcuda(e, "cudaMemcpy");
    b->inputs_dirty = false;
    return CP3_OK;
}

cp3::BatchPrepArgs prep_args(cp3_batch* b, int k) {
    cp3::BatchPrepArgs a{};
    a.grids = b->d_grids.p;
    a.eblk = b->d_eblk.p + b->chunk_eblk[k];
    a.cblk = b->d_cblk.p + b->chunk_cblk[k];
    a.n_eblk = b->chunk_eblk[k + 1] - b->chunk_eblk[k];
    a.n_cblk = b->chunk_cblk[k + 1] - b->chunk_cblk[k];
    a.eb = b->eb;
    a.energies = b->d_en.p;
    a.cosines = b->d_cos.p;
    a.maxl = b->d_maxl.p;
    a.radii = b->d_radii.p;
    a.rhoye = b->d_rhoye.p;
    a.height_cm = b->height_cm;
    a.nl = b->nl;
    a.nl_pad = b->nl_pad;
    a.te = b->te;
    a.tab = b->d_tab.p;
    a.pe = b->d_pe.p;
    a.len = b->d_len.p;
    a.n_sets = b->n_sets;
    a.tab_words = (long long)(b->d_tab.n / (b->mixed ? 4 : 8));
    a.pe_words = (long long)(b->d_pe.n / (b->mixed ? 4 : 8));
    a.len_entries = (long long)(b->d_len.n / 8);
    return a;
}

cp3::BatchPropArgs prop_args(cp3_batch* b, int k) {
    cp3::BatchPropArgs a{};
    a.grids = b->d_grids.p;
    a.items = b->d_items.p + b->chunk_items[k];
    a.n_items = b->chunk_items[k + 1] - b->chunk_items[k];
    a.counter = b->d_counter.p + k;
    a.tab = b->d_tab.p;
    a.pe = b->d_pe.p;
    a.len = b->d_len.p;
    a.maxl = b->d_maxl.p;
    a.ptab = b->d_ptab.p;
    a.out = b->d_out.p;
    a.nl = b->nl;
    a.nl_pad = b->nl_pad;
    a.cchunk = b->cchunk;
    a.n_sets = b->n_sets;
    a.tab_words = (long long)(b->d_tab.n / (b->mixed ? 4 : 8));
    a.pe_words = (long long)(b->d_pe.n / (b->mixed ? 4 : 8));
    a.len_entries = (long long)(b->d_len.n / 8);
    a.out_elems = (long long)(b->d_out.n / b->elem());
    return a;
}

// Capture: counter reset, then per chunk k a prep launch on a side stream and
// the persistent propagate of chunk k on the main stream after it, so that
// chunk k + 1's FP64 prep overlaps chunk k's propagation.
// Blocks per SM of the looping prep launches (measured on the 1024-set batch:
// 2 leave the prep exposed, 55.0 ms per step; 4 51.6 ms; 8 51.9 ms; one block
// per item, about 100,000 per chunk, 52.0 ms).
constexpr int kPrepBlocksPerSM = 4;

int capture(cp3_batch* b) {
    drop_graph(b);
    const int K = b->n_chunks;
    cudaStream_t cs = nullptr, side = nullptr;
    std::vector<cudaEvent_t> evs(K + 2, nullptr);
    // The propagate launches get the higher priority: the block scheduler then
    // dispatches a chunk's persistent wave first and the next chunk's prep
    // blocks (many small FP64 blocks) only into what the wave leaves free,
    // instead of the prep flooding the SMs ahead of the propagation.
    int lo_prio = 0, hi_prio = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (!e) e = cudaStreamCreateWithPriority(&cs, cudaStreamNonBlocking, hi_prio);
    if (!e) e = cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, lo_prio);
    for (int k = 0; k < K + 2 && !e; k++) e = cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming);
    auto cleanup = [&]() {
        for (cudaEvent_t ev : evs)
            if (ev) cudaEventDestroy(ev);
        if (side) cudaStreamDestroy(side);
        if (cs) cudaStreamDestroy(cs);
    };
    if (e) {
        cleanup();
        return bcuda(e, "graph capture set-up");
    }
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    bool capturing = !e;
    // Chunk k's propagation waits for its prep and for chunk k - 1's
    // propagation (one stream): while it runs, chunk k + 1's prep fills the
    // room its persistent wave leaves on every SM.  Letting chunk k + 1's
    // propagation start early instead (a second stream) hands that room to
    // propagate blocks and measured no faster.
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int prep_grid = std::max(1, sms) * kPrepBlocksPerSM;
    if (!e) e = cudaMemsetAsync(b->d_counter.p, 0, sizeof(int) * std::max(1, K), cs);
    if (!e) e = cudaEventRecord(evs[K], cs);  // fork
    if (!e) e = cudaStreamWaitEvent(side, evs[K], 0);
    for (int k = 0; k < K && !e; k++) {
        e = cp3::batch_prep_launch(b->mixed, prep_args(b, k), side, prep_grid);
        if (!e) e = cudaEventRecord(evs[k], side);
        if (!e) e = cudaStreamWaitEvent(cs, evs[k], 0);
        const int n_items = b->chunk_items[k + 1] - b->chunk_items[k];
        if (!e && n_items > 0)
            e = cp3::batch_launch(b->mixed, b->te, prop_args(b, k), b->groups, b->smem, std::min(b->blocks, n_items),
                                  cs);
    }
    if (!e) e = cudaEventRecord(evs[K + 1], side);  // join
    if (!e) e = cudaStreamWaitEvent(cs, evs[K + 1], 0);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = capturing ? cudaStreamEndCapture(cs, &g) : cudaSuccess;
    cleanup();
    if (e || e2) {
        if (g) cudaGraphDestroy(g);
        return bcuda(e ? e : e2, "graph capture");
    }
    b->graph = g;
    if ((e = cudaGraphInstantiate(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority))) {
        drop_graph(b);
        return bcuda(e, "cudaGraphInstantiate");
    }
    return CP3_OK;
}

int ready(cp3_batch* b, int type) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (!b->has_grids) return bfail(CP3_ERR_STATE, "batch: grids were not set");
    if (!b->has_params) return bfail(CP3_ERR_STATE, "batch: parameters were not set");
    if (!b->has_density) return bfail(CP3_ERR_STATE, "batch: density was not set");
    if (!b->has_height) return bfail(CP3_ERR_STATE, "batch: production height was not set");
    if (type != CP3_NEUTRINO && type != CP3_ANTINEUTRINO) return bfail(CP3_ERR_ARGUMENT, "unknown neutrino type");
    int rc;
    if (b->inputs_dirty && (rc = upload_inputs(b))) return rc;
    if (b->layout_dirty && (rc = build_layout(b))) return rc;
    if (type != b->type) {
        b->type = type;
        b->desc_dirty = true;
    }
    if (b->desc_dirty && (rc = upload_descriptors(b))) return rc;
    if (!b->exec && (rc = capture(b))) return rc;
    return CP3_OK;
}

}  // namespace

extern "C" {

int cp3_batch_create(cp3_batch** out, int device_id, int precision, int n_sets, const int* n_cosines,
                     const int* n_energies) {
    if (!out) return bfail(CP3_ERR_ARGUMENT, "cp3_batch_create: null output pointer");
    *out = nullptr;
    if (n_sets < 0 || (n_sets > 0 && (!n_cosines || !n_energies)))
        return bfail(CP3_ERR_ARGUMENT, "cp3_batch_create: bad set list");
    if (precision != CP3_PRECISION_FP64 && precision != CP3_PRECISION_MIXED)
        return bfail(CP3_ERR_ARGUMENT, "cp3_batch_create: unknown precision");
    if (device_id < 0 || device_id >= cp3_device_count()) return bfail(CP3_ERR_NO_DEVICE, "No GPU found");
    Guard g(device_id);
    if (g.err) return bcuda(g.err, "cudaSetDevice");
    cp3_batch* b = new cp3_batch();
    b->device = device_id;
    b->mixed = precision == CP3_PRECISION_MIXED;
    b->n_sets = n_sets;
    if (!b->mixed) {
        b->te = 64;
        b->groups = 2;
    }
    for (int s = 0; s < n_sets; s++) {
        if (n_cosines[s] < 0 || n_energies[s] < 0) {
            delete b;
            return bfail(CP3_ERR_ARGUMENT, "cp3_batch_create: negative grid size");
        }
        b->n_cos.push_back(n_cosines[s]);
        b->n_en.push_back(n_energies[s]);
        b->cos_off.push_back(b->total_cos);
        b->en_off.push_back(b->total_en);
        b->out_off.push_back(b->total_out);
        b->total_cos += n_cosines[s];
        b->total_en += n_energies[s];
        b->total_out += 9LL * n_cosines[s] * n_energies[s];
    }
    b->out_off.push_back(b->total_out);
    b->cosines.assign(b->total_cos, 0.0);
    b->energies.assign(b->total_en, 1.0);
    b->maxl.assign(b->total_cos, 0);
    b->params.assign(6 * (size_t)n_sets, 0.0);
    b->scale.assign(n_sets, 1.0);
    cudaError_t e;
    auto bail = [&](cudaError_t err, const char* w) {
        int rc = bcuda(err, w);
        cp3_batch_destroy(b);
        return rc;
    };
    if ((e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking))) return bail(e, "cudaStreamCreate");
    b->stream = b->own;
    if ((e = b->d_out.ensure((size_t)b->total_out * b->elem()))) return bail(e, "cudaMalloc(results)");
    if ((e = b->d_counter.ensure(1))) return bail(e, "cudaMalloc");
    if ((e = cudaEventCreate(&b->ev[0])) || (e = cudaEventCreate(&b->ev[1]))) return bail(e, "cudaEventCreate");
    std::vector<int4> tab(cp3::kPhaseTabN + 1);
    cp3::fill_phase_table(b->mixed, tab.data());
    if ((e = b->d_ptab.ensure(tab.size())) ||
        (e = cudaMemcpy(b->d_ptab.p, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice)))
        return bail(e, "phase table");
    *out = b;
    return CP3_OK;
}

int cp3_batch_destroy(cp3_batch* b) {
    if (!b) return CP3_OK;
    Guard g(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (auto& e : b->ev)
        if (e) cudaEventDestroy(e);
    b->d_cos.release();
    b->d_en.release();
    b->d_radii.release();
    b->d_rhoye.release();
    b->d_maxl.release();
    b->d_counter.release();
    b->d_grids.release();
    b->d_eblk.release();
    b->d_cblk.release();
    b->d_items.release();
    b->d_ptab.release();
    b->d_tab.release();
    b->d_pe.release();
    b->d_len.release();
    b->d_out.release();
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return CP3_OK;
}

int cp3_batch_set_grids(cp3_batch* b, const double* cosines, const double* energies) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if ((b->total_cos && !cosines) || (b->total_en && !energies)) return bfail(CP3_ERR_ARGUMENT, "null grid array");
    for (long long i = 0; i < b->total_cos; i++)
        if (!(cosines[i] >= -1.0 && cosines[i] <= 1.0))
            return bfail(CP3_ERR_ARGUMENT, "setCosineList: cosines must lie in [-1, 1]");
    for (long long i = 0; i < b->total_en; i++)
        if (!(energies[i] > 0.0) || !std::isfinite(energies[i]))
            return bfail(CP3_ERR_ARGUMENT, "setEnergyList: energies must be finite and positive");
    b->cosines.assign(cosines, cosines + b->total_cos);
    b->energies.assign(energies, energies + b->total_en);
    compute_maxl(b);
    b->has_grids = true;
    b->inputs_dirty = true;
    b->layout_dirty = true;  // work-item costs follow the layer counts
    return CP3_OK;
}

int cp3_batch_set_parameters(cp3_batch* b, const double* params) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (b->n_sets && !params) return bfail(CP3_ERR_ARGUMENT, "null parameter array");
    for (long long i = 0; i < 6LL * b->n_sets; i++)
        if (!std::isfinite(params[i])) return bfail(CP3_ERR_ARGUMENT, "batch: parameters must be finite");
    b->params.assign(params, params + 6 * (size_t)b->n_sets);
    b->has_params = true;
    b->desc_dirty = true;
    return CP3_OK;
}

int cp3_batch_set_density(cp3_batch* b, const double* radii, const double* rhos, const double* ye, int n,
                          const double* scale) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (n <= 0) return bfail(CP3_ERR_ARGUMENT, "setDensity : vectors must not be empty");
    if (!radii || !rhos) return bfail(CP3_ERR_ARGUMENT, "setDensity : null array");
    if (n > CP3_MAX_ROWS) return bfail(CP3_ERR_LIMIT, "setDensity : more than 64 rows");
    // the single-grid handle's ordering and checks (propagator.hpp:117-161)
    cp3::BodyRow rows[CP3_MAX_ROWS];
    if (const char* msg = cp3::order_body(radii, rhos, ye, n, rows)) return bfail(CP3_ERR_ARGUMENT, msg);
    for (int s = 0; scale && s < b->n_sets; s++)
        if (!(scale[s] >= 0.0) || !std::isfinite(scale[s]))
            return bfail(CP3_ERR_ARGUMENT, "batch: density scales must be finite and >= 0");
    b->radii.resize(n);
    b->rhos.resize(n);
    b->ye.resize(n);
    b->coslimit.resize(n);
    for (int i = 0; i < n; i++) {
        b->radii[i] = rows[i].radius;
        b->rhos[i] = rows[i].rho;
        b->ye[i] = rows[i].ye;
        b->coslimit[i] = rows[i].coslimit;
    }
    if (scale)
        b->scale.assign(scale, scale + b->n_sets);
    else
        b->scale.assign(b->n_sets, 1.0);
    compute_maxl(b);
    b->has_density = true;
    b->inputs_dirty = true;
    b->layout_dirty = true;
    return CP3_OK;
}

int cp3_batch_set_production_height(cp3_batch* b, double km) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (!std::isfinite(km)) return bfail(CP3_ERR_ARGUMENT, "setProductionHeight: height must be finite");
    b->height_cm = km * 100000.0;
    b->has_height = true;
    drop_graph(b);  // the height is a kernel argument of the captured prep launch
    return CP3_OK;
}

int cp3_batch_set_stream(cp3_batch* b, void* s) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    b->stream = s ? (cudaStream_t)s : b->own;
    return CP3_OK;
}

int cp3_batch_set_launch_shape(cp3_batch* b, int te, int groups, int cchunk) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if ((te != 32 && te != 64 && te != 128) || groups < 1 || te * groups > cp3::propagate_max_threads(b->mixed) ||
        cchunk < 1 || cchunk > 1024)
        return bfail(CP3_ERR_ARGUMENT, "batch: unsupported launch shape");
    b->te = te;
    b->groups = groups;
    b->cchunk = cchunk;
    b->layout_dirty = true;
    return CP3_OK;
}

int cp3_batch_get_launch_shape(cp3_batch* b, int* te, int* groups, int* cchunk, int* blocks) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (te) *te = b->te;
    if (groups) *groups = b->groups;
    if (cchunk) *cchunk = b->cchunk;
    if (blocks) *blocks = b->blocks;
    return CP3_OK;
}

int cp3_batch_calculate_async(cp3_batch* b, int type) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    Guard g(b->device);
    cudaGetLastError();  // a failed earlier call must not be reported by the checks below
    if (int rc = ready(b, type)) return rc;
    cudaError_t e;
    if ((e = cudaEventRecord(b->ev[0], b->stream))) return bcuda(e, "cudaEventRecord");
    if ((e = cudaGraphLaunch(b->exec, b->stream))) return bcuda(e, "cudaGraphLaunch");
    if ((e = cudaEventRecord(b->ev[1], b->stream))) return bcuda(e, "cudaEventRecord");
    return CP3_OK;
}

int cp3_batch_wait(cp3_batch* b) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    Guard g(b->device);
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e) return bcuda(e, "cudaStreamSynchronize");
    float ms = 0;
    if (cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]) == cudaSuccess) b->last_ms = ms;
    // checked build: this file's kernels and the single-grid kernels of the
    // sequential path (nothing to read otherwise)
    if (cp3::kChecked) {
        cp3::CheckRecord r{}, r2{};
        if ((e = cp3::check_take(&r)) || (e = cp3::kernels_check_take(&r2))) return bcuda(e, "bounds-check record");
        if (int rc = cp3::check_status(r.count ? r : r2)) return rc;
    }
    return CP3_OK;
}

int cp3_batch_calculate(cp3_batch* b, int type) {
    int rc = cp3_batch_calculate_async(b, type);
    return rc ? rc : cp3_batch_wait(b);
}

// The same work as separate launches: for every set, one prep and one
// propagate launch of the single-grid kernels (two launches per set).
int cp3_batch_calculate_sequential(cp3_batch* b, int type) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    Guard g(b->device);
    cudaGetLastError();
    if (int rc = ready(b, type)) return rc;
    cudaError_t e;
    if ((e = cudaEventRecord(b->ev[0], b->stream))) return bcuda(e, "cudaEventRecord");
    const size_t word = b->mixed ? 4 : 8;
    const size_t smem = cp3::propagate_smem_bytes(b->mixed, b->te, b->nl, b->nl_pad, b->cchunk);
    for (int s = 0; s < b->n_sets; s++) {
        const cp3::BatchGrid& gr = b->grids[s];
        if (gr.n_cos == 0 || gr.n_en == 0) continue;
        cp3::PrepArgs pa{};
        pa.pb.n_cos = gr.n_cos;
        pa.pb.n_en = gr.n_en;
        pa.pb.n_en_pad = gr.n_en_pad;
        pa.pb.te = b->te;
        pa.pb.nl = b->nl;
        pa.pb.nl_pad = b->nl_pad;
        pa.pb.energies = b->d_en.p + gr.en_off;
        pa.pb.cosines = b->d_cos.p + gr.cos_off;
        pa.pb.maxlayers = b->d_maxl.p + gr.cos_off;
        pa.pb.radii = b->d_radii.p;
        pa.pb.rhoye = b->d_rhoye.p + gr.rhoye_off;
        pa.pb.height_cm = b->height_cm;
        pa.osc = gr.osc;
        pa.tab = b->d_tab.p + gr.tab_off * word;
        pa.pe = b->d_pe.p + gr.pe_off * word;
        pa.len = b->d_len.p + gr.len_off * 8;
        if ((e = cp3::launch_prep(b->mixed, pa, b->stream))) return bcuda(e, "prep kernel");
        cp3::PropArgs ka{};
        ka.tab = pa.tab;
        ka.pe = pa.pe;
        ka.len = pa.len;
        ka.maxl = pa.pb.maxlayers;
        ka.ptab = b->d_ptab.p;
        ka.out = b->d_out.p + gr.out_off * b->elem();
        ka.n_cos = gr.n_cos;
        ka.n_en = gr.n_en;
        ka.n_en_pad = gr.n_en_pad;
        ka.nl = b->nl;
        ka.nl_pad = b->nl_pad;
        ka.cchunk = b->cchunk;
        if ((e = cp3::launch_propagate(b->mixed, ka, b->te, b->groups, smem, b->stream)))
            return bcuda(e, "propagate kernel");
    }
    if ((e = cudaEventRecord(b->ev[1], b->stream))) return bcuda(e, "cudaEventRecord");
    return cp3_batch_wait(b);
}

int cp3_batch_last_ms(cp3_batch* b, float* ms) {
    if (!b || !ms) return bfail(CP3_ERR_ARGUMENT, "null argument");
    *ms = b->last_ms;
    return CP3_OK;
}

int cp3_batch_launch_count(cp3_batch* b, int type, int* launches) {
    if (!b || !launches) return bfail(CP3_ERR_ARGUMENT, "null argument");
    Guard g(b->device);
    if (g.err) return bcuda(g.err, "cudaSetDevice");
    if (int rc = ready(b, type)) return rc;  // the layout the graph is captured from
    int n = b->n_chunks;                      // one prep launch per chunk
    for (int k = 0; k < b->n_chunks; k++) n += (b->chunk_items[k + 1] > b->chunk_items[k]);
    *launches = n;
    return CP3_OK;
}

int cp3_batch_result_offsets(cp3_batch* b, long long* offsets) {
    if (!b || !offsets) return bfail(CP3_ERR_ARGUMENT, "null argument");
    std::copy(b->out_off.begin(), b->out_off.end(), offsets);
    return CP3_OK;
}

int cp3_batch_result_device_ptr(cp3_batch* b, void** dptr) {
    if (!b || !dptr) return bfail(CP3_ERR_ARGUMENT, "null argument");
    *dptr = b->d_out.p;
    return CP3_OK;
}

int cp3_batch_copy_results_to_host(cp3_batch* b, void* dst, size_t bytes) {
    if (!b || !dst) return bfail(CP3_ERR_ARGUMENT, "null argument");
    const size_t need = (size_t)b->total_out * b->elem();
    if (bytes < need) return bfail(CP3_ERR_ARGUMENT, "batch: destination too small");
    if (need == 0) return CP3_OK;
    Guard g(b->device);
    cudaError_t e = cudaMemcpyAsync(dst, b->d_out.p, need, cudaMemcpyDeviceToHost, b->stream);
    if (!e) e = cudaStreamSynchronize(b->stream);
    return e ? bcuda(e, "cudaMemcpyAsync(results)") : CP3_OK;
}

int cp3_batch_get_maxlayers(cp3_batch* b, int* out, long long n) {
    if (!b || (n && !out) || n != b->total_cos) return bfail(CP3_ERR_ARGUMENT, "batch: n must equal the total cosines");
    std::copy(b->maxl.begin(), b->maxl.end(), out);
    return CP3_OK;
}

// Launch-shape search: every supported (te, groups, cchunk), each timed on
// `reps` graph launches of the whole batch; the fastest is kept.
int cp3_batch_autotune(cp3_batch* b, int type, int reps, int* te_out, int* groups_out, int* cchunk_out,
                       float* best_ms) {
    if (!b) return bfail(CP3_ERR_ARGUMENT, "null batch handle");
    if (reps < 1) reps = 1;
    const int tes[3] = {32, 64, 128};
    const int chunks[4] = {8, 16, 32, 64};
    float best = 1e30f;
    int bt = b->te, bg = b->groups, bc = b->cchunk;
    for (int te : tes)
        for (int groups = 1; te * groups <= cp3::propagate_max_threads(b->mixed); groups *= 2) {
            if (te * groups < 64) continue;
            for (int cc : chunks) {
                if (cc < groups) continue;
                if (cp3_batch_set_launch_shape(b, te, groups, cc)) continue;
                int rc = cp3_batch_calculate(b, type);  // warm-up (builds layout and graph)
                if (rc == CP3_ERR_LIMIT) continue;
                if (rc) return rc;
                float tot = 0;
                for (int r = 0; r < reps; r++) {
                    if ((rc = cp3_batch_calculate(b, type))) return rc;
                    tot += b->last_ms;
                }
                const float ms = tot / reps;
                if (ms < best) {
                    best = ms;
                    bt = te;
                    bg = groups;
                    bc = cc;
                }
            }
        }
    if (int rc = cp3_batch_set_launch_shape(b, bt, bg, bc)) return rc;
    if (te_out) *te_out = bt;
    if (groups_out) *groups_out = bg;
    if (cchunk_out) *cchunk_out = bc;
    if (best_ms) *best_ms = best;
    return CP3_OK;
}

}  // extern "C"

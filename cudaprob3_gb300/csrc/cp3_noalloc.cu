// One calculation that allocates nothing: cp3_propagate_noalloc.
//
// Some callers cannot call cudaMalloc.  A framework whose caching allocator
// owns (nearly) all device memory leaves no room for allocations made behind
// its back, and every cudaFree synchronises the whole device.  A fitter that
// evaluates thousands of parameter points per second cannot take that
// synchronisation inside its loop.  A plugin that a host application hands
// only device pointers and a stream is not allowed to own device memory at
// all.  For such callers this entry point runs the single-grid calculation
// (precompute, then propagation) on the caller's device pointers and stream,
// with its scratch tables in a file-scope __device__ array instead of
// per-handle allocations.
//
// The array is sized for grids up to kNoAllocMaxCosines x kNoAllocMaxEnergies
// and kNoAllocMaxRows density rows, in either precision (about 14 MB); every
// GPU that loads the library holds it until the process exits.  The first call
// on a device sets that device up (the array's device address, and the two
// phase tables, written once from the same host function the handle path
// uses, so both paths compute with the same bits).  Every later call rewrites
// each region it reads, so no call depends on the previous one's data; calls
// whose work overlaps on the GPU (other streams, other host threads) race on
// the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "cudaprob3_gb300.h"
#include "cp3_launch.h"
#include "cp3_tile.cuh"

namespace cp3 {

constexpr int kNoAllocMaxCosines = CP3_NOALLOC_MAX_COSINES;
constexpr int kNoAllocMaxEnergies = CP3_NOALLOC_MAX_ENERGIES;
constexpr int kNoAllocMaxRows = CP3_NOALLOC_MAX_ROWS;
constexpr int kNoAllocMaxLayers = kNoAllocMaxRows + 1;  // vacuum + rows
constexpr int kNoAllocLayersPad = (kNoAllocMaxLayers + 1) / 2 * 2;

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
// regions (bytes) for the largest problem; FP64 words are the larger ones
constexpr size_t kNaTab = align256((size_t)kNoAllocMaxEnergies * kNoAllocMaxLayers * kFp64Words * 8);
constexpr size_t kNaPe = align256((size_t)kPerEWords * kNoAllocMaxEnergies * 8);
constexpr size_t kNaLen = align256((size_t)kNoAllocMaxCosines * kNoAllocLayersPad * 8);
constexpr size_t kNaMaxl = align256((size_t)kNoAllocMaxCosines * 4);
constexpr size_t kNaPhase = align256((size_t)kPhaseTabBytes);  // one table per precision
constexpr size_t kNaBody = align256((size_t)2 * kNoAllocMaxLayers * 8);  // radii, rho*Ye
constexpr size_t kNaBytes = kNaTab + kNaPe + kNaLen + kNaMaxl + 2 * kNaPhase + kNaBody;

// offsets of the regions in the array
constexpr size_t kOffPe = kNaTab;
constexpr size_t kOffLen = kOffPe + kNaPe;
constexpr size_t kOffMaxl = kOffLen + kNaLen;
constexpr size_t kOffPhaseMixed = kOffMaxl + kNaMaxl;  // written once per device at set-up
constexpr size_t kOffPhaseFp64 = kOffPhaseMixed + kNaPhase;  // written once per device at set-up
constexpr size_t kOffBody = kOffPhaseFp64 + kNaPhase;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NoAllocBody {
    int n;                              // rows
    double radii[kNoAllocMaxRows];      // outside-in
    double rhoye[kNoAllocMaxLayers];    // layer 0 = vacuum
    double coslimit[kNoAllocMaxRows];   // propagator.hpp:149-158
};

// Writes the layer radii and densities and the layer count of every cosine
// (propagator.hpp:301-307) into the scratch.
__global__ void noalloc_setup_kernel(NoAllocBody body, const double* cosines, int n_cos, double* radii,
                                     double* rhoye, int* maxl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < body.n) radii[CP3_IX(kSiteNoAlloc, t, kNoAllocMaxLayers)] = body.radii[t];
    if (t <= body.n) rhoye[CP3_IX(kSiteNoAlloc, t, kNoAllocMaxLayers)] = body.rhoye[t];
    if (t < n_cos) {
        const double cz = cosines[t];
        int cnt = 0;
        for (int i = 0; i < body.n; i++) cnt += (cz < body.coslimit[i]);
        maxl[CP3_IX(kSiteNoAlloc, t, kNoAllocMaxCosines)] = cnt;
    }
}

}  // namespace cp3

namespace {

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[256] = {};  // device address of the array, per device id; null until set up

int nfail(int code, const std::string& m) {
    cp3::set_last_error(m);
    return code;
}

// Set-up of the current device `dev` (called under g_noalloc_mutex): the
// device address of the scratch array -- its host-side name is only a
// stand-in and must never be passed to a kernel -- and the phase tables of
// both precisions, filled by the same host function as a handle's table and
// copied once (synchronously) into their regions.
cudaError_t noalloc_setup_device(int dev) {
    void* base = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&base, cp3::g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    int4 tab[cp3::kPhaseTabN + 1];
    unsigned char* sc = (unsigned char*)base;
    cp3::fill_phase_table(true, tab);
    if ((e = cudaMemcpy(sc + cp3::kOffPhaseMixed, tab, sizeof tab, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    cp3::fill_phase_table(false, tab);
    if ((e = cudaMemcpy(sc + cp3::kOffPhaseFp64, tab, sizeof tab, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    g_noalloc_ptr[dev] = base;
    return cudaSuccess;
}

}  // namespace

extern "C" int cp3_propagate_noalloc(int precision, int type, const double* d_cosines, int n_cosines,
                                     const double* d_energies, int n_energies, const double* radii,
                                     const double* rhos, const double* ye, int n_rows, double theta12,
                                     double theta13, double theta23, double dcp, double dm12sq, double dm23sq,
                                     double height_km, void* d_out, void* stream) {
    using namespace cp3;
    if (precision != CP3_PRECISION_FP64 && precision != CP3_PRECISION_MIXED)
        return nfail(CP3_ERR_ARGUMENT, "propagate_noalloc: unknown precision");
    if (type != CP3_NEUTRINO && type != CP3_ANTINEUTRINO)
        return nfail(CP3_ERR_ARGUMENT, "propagate_noalloc: unknown neutrino type");
    if (n_cosines < 0 || n_energies < 0 || n_cosines > kNoAllocMaxCosines || n_energies > kNoAllocMaxEnergies)
        return nfail(CP3_ERR_LIMIT, "propagate_noalloc: grid larger than " + std::to_string(kNoAllocMaxCosines) +
                                        " cosines x " + std::to_string(kNoAllocMaxEnergies) + " energies");
    if (n_rows <= 0) return nfail(CP3_ERR_ARGUMENT, "setDensity : vectors must not be empty");
    if (n_rows > kNoAllocMaxRows)
        return nfail(CP3_ERR_LIMIT, "propagate_noalloc: more than " + std::to_string(kNoAllocMaxRows) + " density rows");
    if (!radii || !rhos || (n_cosines && !d_cosines) || (n_energies && !d_energies) ||
        (n_cosines && n_energies && !d_out))
        return nfail(CP3_ERR_ARGUMENT, "propagate_noalloc: null pointer");
    const double par[7] = {theta12, theta13, theta23, dcp, dm12sq, dm23sq, height_km};
    for (double v : par)
        if (!std::isfinite(v)) return nfail(CP3_ERR_ARGUMENT, "propagate_noalloc: parameters must be finite");
    // setDensity (propagator.hpp:117-161), the same checks and order as cp3_set_density
    BodyRow rows[kNoAllocMaxRows];
    if (const char* msg = order_body(radii, rhos, ye, n_rows, rows)) return nfail(CP3_ERR_ARGUMENT, msg);
    NoAllocBody body{};
    body.n = n_rows;
    body.rhoye[0] = 0.0;
    for (int i = 0; i < n_rows; i++) {
        body.radii[i] = rows[i].radius;
        body.rhoye[i + 1] = rows[i].rho * rows[i].ye;
        body.coslimit[i] = rows[i].coslimit;
    }
    if (n_cosines == 0 || n_energies == 0) return CP3_OK;

    // set-up once per device, with that device current
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nfail(CP3_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 256) return nfail(CP3_ERR_NO_DEVICE, "propagate_noalloc: device id out of range");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev] && (e = noalloc_setup_device(dev)) != cudaSuccess)
            return nfail(CP3_ERR_CUDA, std::string("propagate_noalloc set-up: ") + cudaGetErrorString(e));
        base = g_noalloc_ptr[dev];
    }
    const bool mixed = precision == CP3_PRECISION_MIXED;
    unsigned char* sc = (unsigned char*)base;
    void* tab = sc;
    void* pe = sc + kOffPe;
    void* len = sc + kOffLen;
    int* maxl = (int*)(sc + kOffMaxl);
    const int4* ptab = (const int4*)(sc + (mixed ? kOffPhaseMixed : kOffPhaseFp64));
    double* d_radii = (double*)(sc + kOffBody);
    double* d_rhoye = d_radii + kNoAllocMaxLayers;

    cudaStream_t s = (cudaStream_t)stream;
    cudaGetLastError();  // an earlier failed call must not be reported by the checks below
    const int nl = n_rows + 1;
    const int nl_pad = (nl + 1) / 2 * 2;
    // the default launch shape of a handle (cp3_create), so that both paths
    // run the same kernels on the same tiles
    const int te = 64, groups = mixed ? 4 : 2, cchunk = 32;
    const int n_en_pad = (n_energies + te - 1) / te * te;
    {
        const int n = std::max(n_cosines, n_rows + 1);
        noalloc_setup_kernel<<<(n + 255) / 256, 256, 0, s>>>(body, d_cosines, n_cosines, d_radii, d_rhoye, maxl);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return nfail(CP3_ERR_CUDA, std::string("setup kernel: ") + cudaGetErrorString(e));
    }
    PrepArgs pa{};
    pa.pb.n_cos = n_cosines;
    pa.pb.n_en = n_energies;
    pa.pb.n_en_pad = n_en_pad;
    pa.pb.te = te;
    pa.pb.nl = nl;
    pa.pb.nl_pad = nl_pad;
    pa.pb.energies = d_energies;
    pa.pb.cosines = d_cosines;
    pa.pb.maxlayers = maxl;
    pa.pb.radii = d_radii;
    pa.pb.rhoye = d_rhoye;
    // a handle's height after setProductionHeight (propagator.hpp:279-286)
    pa.pb.height_cm = height_km * 100000.0;
    fill_osc_params(pa.osc, theta12, theta13, theta23, dcp, dm12sq, dm23sq, type == CP3_ANTINEUTRINO);
    pa.tab = tab;
    pa.pe = pe;
    pa.len = len;
    if ((e = launch_prep(mixed, pa, s)) != cudaSuccess)
        return nfail(CP3_ERR_CUDA, std::string("prep kernel: ") + cudaGetErrorString(e));
    PropArgs ka{};
    ka.tab = tab;
    ka.pe = pe;
    ka.len = len;
    ka.maxl = maxl;
    ka.ptab = ptab;
    ka.out = d_out;
    ka.n_cos = n_cosines;
    ka.n_en = n_energies;
    ka.n_en_pad = n_en_pad;
    ka.nl = nl;
    ka.nl_pad = nl_pad;
    ka.cchunk = cchunk;
    const size_t smem = propagate_smem_bytes(mixed, te, nl, nl_pad, cchunk);
    if ((e = launch_propagate(mixed, ka, te, groups, smem, s)) != cudaSuccess)
        return nfail(CP3_ERR_CUDA, std::string("propagate kernel: ") + cudaGetErrorString(e));
    if (kChecked) {
        // the bounds-checked build waits for the call and reports its failed
        // checks (the set-up kernel's, and the prep and propagate kernels')
        CheckRecord r{}, r2{};
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess || (e = check_take(&r)) != cudaSuccess ||
            (e = kernels_check_take(&r2)) != cudaSuccess)
            return nfail(CP3_ERR_CUDA, std::string("bounds-check record: ") + cudaGetErrorString(e));
        if (int rc = check_status(r.count ? r : r2)) return rc;
    }
    return CP3_OK;
}

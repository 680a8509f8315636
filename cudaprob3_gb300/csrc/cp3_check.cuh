// Bounds checks of the debug build (compiled with -DCP3_CHECK into
// libcudaprob3_gb300_check.so; without it every check below compiles to the
// bare index).
//
// The reference indexes its device arrays unchecked (physics.hpp:689-696,
// cudapropagator.cuh:204-209), and no sanitizer runs on the GPUs this library
// is tested on, so the debug build checks each index itself: before a kernel
// touches a shared- or global-memory buffer at index i, CP3_IX(site, i, n)
// compares i with the buffer's extent n.  An index outside [0, n) is recorded
// in the check record of its translation unit -- the first failure's site,
// index and extent, and a count of all failures -- and replaced by 0, so the
// access stays inside the buffer.  No kernel traps or stops early because of a
// check; its results are then wrong, and the host says so: after each
// calculation it reads and clears the record and returns CP3_ERR_CHECK with
// the site and the index in cp3_last_error().
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

namespace cp3 {

struct CheckRecord {
    unsigned int count;  // failed checks since the last read
    int site;            // CheckSite of the first failure
    long long index;     // its index
    long long bound;     // and the extent it had to stay below
};

// Where an index is checked: kernel and buffer.
enum CheckSite : int {
    kSiteNone = 0,
    kSiteTileTab,       // process_tile: global energy-tile table, staged copy
    kSiteTilePe,        // process_tile: global per-energy table
    kSiteTileLen,       // process_tile: global segment lengths of the cosine chunk
    kSiteTileMaxl,      // process_tile: global layer counts
    kSiteTileLayers,    // process_tile: a pair's layer count against the layer table
    kSiteTileChunk,     // process_tile: cosine row against the staged chunk
    kSiteTileOut,       // process_tile: result planes
    kSiteTileFlux,      // process_tile: fused-rate flux
    kSiteTileHist,      // process_tile: fused-rate histogram bin
    kSiteTileHeights,   // process_tile: per-height atmosphere lengths
    kSitePhaseTable,    // phase evaluation: index into the 257-entry table
    kSitePrepEnergy,    // prep: energy list
    kSitePrepLayer,     // prep: layer against the density rows
    kSitePrepTab,       // prep: energy-tile table entry
    kSitePrepPe,        // prep: per-energy table entry
    kSitePrepLen,       // prep: segment-length entry
    kSitePrepShared,    // prep: eigenvectors in shared memory
    kSiteBatchItem,     // batch propagate: work item
    kSiteBatchSet,      // batch: set index of a work item or prep block
    kSiteBatchTile,     // batch propagate: energy tile / cosine range of an item
    kSiteBatchPrep,     // batch prep: energy / cosine of a prep block
    kSiteLLPair,        // log-likelihood pair kernel: bin / partial index
    kSiteLLLayer,       // log-likelihood layer kernel: partial / table index
    kSiteLLPrep,        // log-likelihood prep kernel: table index
    kSiteNoAlloc,       // no-allocation set-up kernel
    kSiteCount
};

inline const char* check_site_name(int site) {
    static const char* const names[kSiteCount] = {
        "none",
        "process_tile: energy-tile table",
        "process_tile: per-energy table",
        "process_tile: segment lengths",
        "process_tile: layer counts",
        "process_tile: layer count vs layer table",
        "process_tile: cosine row vs staged chunk",
        "process_tile: result planes",
        "process_tile: rate flux",
        "process_tile: histogram bin",
        "process_tile: per-height lengths",
        "phase table index",
        "prep: energy list",
        "prep: density layer",
        "prep: energy-tile table",
        "prep: per-energy table",
        "prep: segment lengths",
        "prep: shared eigenvectors",
        "batch propagate: work item",
        "batch: set index",
        "batch propagate: tile range",
        "batch prep: block range",
        "loglik pair kernel",
        "loglik layer kernel",
        "loglik prep kernel",
        "noalloc set-up kernel",
    };
    return (site >= 0 && site < kSiteCount) ? names[site] : "unknown";
}

#ifdef CP3_CHECK
constexpr bool kChecked = true;

// One record per translation unit (internal linkage): the kernels of a .cu
// file write it, and host code of the same file reads it (check_take).
static __device__ CheckRecord g_check_record;

__device__ __forceinline__ long long checked_index(int site, long long i, long long n) {
    if (i >= 0 && i < n) return i;
    if (atomicAdd(&g_check_record.count, 1u) == 0u) {
        g_check_record.site = site;
        g_check_record.index = i;
        g_check_record.bound = n;
    }
    return 0;
}

#define CP3_IX(site, i, n) \
    ((std::decay_t<decltype(i)>)::cp3::checked_index((site), (long long)(i), (long long)(n)))

// The same check as a condition, for a whole range or work item: true when
// 0 <= i < n; a failure is recorded and the caller skips the work.
__device__ __forceinline__ bool check_ok(int site, long long i, long long n) {
    if (i >= 0 && i < n) return true;
    checked_index(site, i, n);
    return false;
}

// Reads and clears this translation unit's record on the current device
// (synchronous; call after the calculation's stream has completed).
static inline cudaError_t check_take(CheckRecord* out) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_check_record, sizeof(CheckRecord));
    if (e != cudaSuccess) return e;
    const CheckRecord zero{};
    return cudaMemcpyToSymbol(g_check_record, &zero, sizeof(CheckRecord));
}
#else
constexpr bool kChecked = false;
#define CP3_IX(site, i, n) (i)
__device__ __forceinline__ constexpr bool check_ok(int, long long, long long) { return true; }
static inline cudaError_t check_take(CheckRecord* out) {
    *out = CheckRecord{};
    return cudaSuccess;
}
#endif

}  // namespace cp3

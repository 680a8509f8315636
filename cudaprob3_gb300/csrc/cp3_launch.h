// Host-side launch interface of the propagator kernels (internal).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>

#include "cp3_check.cuh"
#include "cp3_internal.h"

namespace cp3 {

struct PrepArgs {
    Problem pb;
    OscParams osc;
    void* tab;  // per-(energy, layer) table, tile-major
    void* pe;   // per-energy V_0, V_1
    void* len;  // per-(cosine, layer) lengths
    int n_energy_blocks;  // set by launch_prep
    // production-height average: atmosphere length of every cosine at each height
    const double* heights_cm;  // [n_h] or null
    int n_h;
    void* lenh;                // [n_cos][n_h] float2 hi/lo (mixed) or double
};

struct PropArgs {
    const void* tab;
    const void* pe;
    const void* len;
    const int* maxl;
    const int4* ptab;  // mixed: 257 (Q1.30 cos, Q1.30 sin, float cos, float sin) of 2*pi*j/256
    void* out;
    int n_cos, n_en, n_en_pad, nl, nl_pad, cchunk;
    // fused rates (launch_propagate with rates = true): see TileJob
    const float* flux;
    int flux_mask;
    const int* cbin;
    const int* ebin;
    double* hist;
    int n_cb, n_eb;
    // production-height average (mode kModeHeights): see TileJob
    const void* lenh;
    const void* hw;
    int n_h;
};

size_t propagate_smem_bytes(bool mixed, int te, int nl, int nl_pad, int cchunk);

// Largest dynamic shared memory a block of the current device may opt in to.
int max_dynamic_smem();

// Opts kernel `func` in to max_dynamic_smem() bytes of dynamic shared memory
// on the current device.  A function attribute belongs to one device's
// context, so the opt-in is made once per (kernel, device) -- not once per
// process -- under a lock, so that handles on several devices and several
// host threads may launch the same kernel.
cudaError_t opt_in_max_smem(const void* func);

// Largest block (threads) the propagate kernel of a precision accepts.
inline int propagate_max_threads(bool mixed) { return mixed ? 256 : 128; }
cudaError_t launch_prep(bool mixed, PrepArgs a, cudaStream_t s);
// mode: 0 planes, 1 fused rates, 2 planes averaged over production heights,
// 3 the four planes of the 2x2 flavour block only
cudaError_t launch_propagate(bool mixed, const PropArgs& a, int te, int groups, size_t smem,
                             cudaStream_t s, int mode = 0);

// The 257-entry phase table of the propagate kernels, j = -128..128 at index
// j + 128: mixed (Q1.30 cos, Q1.30 sin, float cos * 2^30, float sin * 2^30)
// of 2*pi*j/256; FP64 (double cos, double sin) in the same 16 bytes.
inline void fill_phase_table(bool mixed, int4* tab) {
    for (int j = -kPhaseTabN / 2; j <= kPhaseTabN / 2; j++) {
        const double ang = kTwoPi * j / kPhaseTabN;
        const double c = std::cos(ang), s = std::sin(ang);
        int4& out = tab[j + kPhaseTabN / 2];
        if (mixed) {
            const float cf = (float)c * 1073741824.0f, sf = (float)s * 1073741824.0f;
            int ci, si;
            std::memcpy(&ci, &cf, 4);
            std::memcpy(&si, &sf, 4);
            out = make_int4((int)std::llround(c * 1073741824.0), (int)std::llround(s * 1073741824.0), ci, si);
        } else {
            const double cs[2] = {c, s};
            std::memcpy(&out, cs, sizeof cs);
        }
    }
}

// One density row after Propagator::setDensity's reordering: outermost first.
struct BodyRow {
    double radius, rho, ye;
    double coslimit;  // cosine below which a trajectory enters this shell
    int row;          // the caller's index of this row
};

// Propagator::setDensity (propagator.hpp:117-161) for n >= 1 rows given in
// either monotone order: checks the values (finite, >= 0, ye in [0, 1]; ye
// may be null for 0.5 everywhere), flips an ascending list to outside-in, and
// forms coslimit[i] = -sqrt(1 - r_i^2 / R^2) with coslimit[0] = 0.  Writes n
// rows into `out` and returns nullptr, or returns the error message (the
// reference's text where it has one) and leaves `out` undefined.
inline const char* order_body(const double* radii, const double* rhos, const double* ye, int n, BodyRow* out) {
    for (int i = 0; i < n; i++) {
        if (!std::isfinite(radii[i]) || !std::isfinite(rhos[i]) || radii[i] < 0.0 || rhos[i] < 0.0)
            return "setDensity : radii and densities must be finite and >= 0";
        if (ye && !(ye[i] >= 0.0 && ye[i] <= 1.0)) return "setDensity : electron fractions must lie in [0, 1]";
    }
    bool flip = false;
    if (n >= 2) {
        const int sign = (radii[1] - radii[0] > 0 ? 1 : -1);
        for (int i = 1; i < n; i++)
            if ((radii[i] - radii[i - 1]) * sign < 0) return "radii order messed up";
        flip = (sign == 1);
    }
    for (int i = 0; i < n; i++) {
        const int s = flip ? n - 1 - i : i;
        out[i].radius = radii[s];
        out[i].rho = rhos[s];
        out[i].ye = ye ? ye[s] : 0.5;
        out[i].row = s;
        double x = -1 * std::sqrt(1 - (out[i].radius * out[i].radius / (kREarth * kREarth)));
        if (i == 0) x = 0;
        out[i].coslimit = x;
    }
    return nullptr;
}

// Message returned by cp3_last_error() on this thread.
void set_last_error(const std::string& msg);

// Checked build: reads and clears the check record of the single-grid
// kernels (prep_kernel, propagate_kernel); an empty record otherwise.
cudaError_t kernels_check_take(CheckRecord* out);

// CP3_OK for an empty record; otherwise CP3_ERR_CHECK with the first failed
// check (site, index, extent) and the count as the last error.
int check_status(const CheckRecord& r);

}  // namespace cp3

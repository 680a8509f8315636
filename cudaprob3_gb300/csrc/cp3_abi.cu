// C ABI of the propagator: host logic of cudaprob3::Propagator<FLOAT_T>
// (propagator.hpp:43-337) and cudaprob3::CudaPropagatorSingle<FLOAT_T>
// (cudapropagator.cuh:39-251), restated with per-handle state and status codes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "cudaprob3_gb300.h"
#include "cp3_launch.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    return fail(CP3_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Makes `dev` current for the scope and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
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

namespace cp3 {
void set_last_error(const std::string& msg) { g_last_error = msg; }

int check_status(const CheckRecord& r) {
    if (r.count == 0) return CP3_OK;
    return fail(CP3_ERR_CHECK, std::string("bounds check failed: ") + check_site_name(r.site) + ", index " +
                                   std::to_string(r.index) + " not in [0, " + std::to_string(r.bound) + ") (" +
                                   std::to_string(r.count) + " failed checks)");
}
}  // namespace cp3

struct cp3_propagator {
    int device = 0;
    int n_cos = 0, n_en = 0;
    bool mixed = false;

    // host state of Propagator (propagator.hpp:317-336)
    std::vector<double> energies, cosines;
    std::vector<int> maxlayers;
    std::vector<double> radii, rhos, ye, coslimit;  // descending radii after setDensity
    double th12 = 0, th13 = 0, th23 = 0, dcp = 0, dm12 = 0, dm23 = 0;
    double height_cm = 0;
    bool has_mns = false, has_masses = false, has_density = false;
    bool has_energy = false;
    bool is_set_cosine = false, is_set_height = false;

    // device state
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf<double> d_energy, d_cosine, d_radii, d_rhoye;
    DevBuf<int> d_maxl;
    DevBuf<unsigned char> d_tab, d_pe, d_len, d_result;
    DevBuf<int4> d_ptab;
    void* ext_result = nullptr;
    size_t ext_bytes = 0;
    void* ext_host = nullptr;  // caller page-locked host buffer behind ext_result (zero-copy)
    bool host_completion = false;  // with ext_host: store the 2x2 block, derive the rest on the host
    bool completion_pending = false;

    // fused event rates
    DevBuf<float> d_flux;
    const float* ext_flux = nullptr;  // caller device flux (instead of d_flux)
    int flux_mask = 0;
    bool has_flux = false, has_bins = false;
    DevBuf<int> d_cbin, d_ebin;
    DevBuf<double> d_hist;
    int n_cb = 0, n_eb = 0;
    const float* rate_flux() const { return ext_flux ? ext_flux : d_flux.p; }

    // production-height distribution (n_h > 1; otherwise the single height_cm)
    std::vector<double> heights_cm, height_w;
    int n_h = 0;
    bool heights_dirty = false;
    DevBuf<double> d_heights;
    DevBuf<unsigned char> d_hw, d_lenh;
    bool maxl_dirty = true, energy_dirty = true, cosine_dirty = true, density_dirty = true;

    // pinned host copy for getProbability (cudapropagator.cuh:73, 168-181)
    void* h_result = nullptr;
    bool results_on_host = false;
    int last_launches = 0;

    // launch shape
    int te = 64, groups = 4, cchunk = 32;

    // optional per-kernel timing
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    size_t elem() const { return mixed ? sizeof(float) : sizeof(double); }
    size_t result_bytes() const { return (size_t)9 * n_cos * n_en * elem(); }
    void* result_ptr() const { return ext_result ? ext_result : (void*)d_result.p; }
};

namespace {

// propagator.hpp:301-307: layers crossed = number of cosine limits above c.
void set_maxlayers(cp3_propagator* p) {
    for (int ic = 0; ic < p->n_cos; ic++) {
        const double c = p->cosines[ic];
        int cnt = 0;
        for (double lim : p->coslimit) cnt += (c < lim);
        p->maxlayers[ic] = cnt;
    }
    p->maxl_dirty = true;
}

int check(cp3_propagator* p) {
    if (!p) return fail(CP3_ERR_ARGUMENT, "null propagator handle");
    return CP3_OK;
}

}  // namespace

namespace {

// The five planes that unitarity fixes, from the four of the 2x2 flavour
// block stored by the kernel (planes in*3+out: rows and columns of the 3x3
// probability matrix sum to one), on the host cores; doubles inside, one
// rounding to the plane type, clamped at zero like the kernel's completion.
template <class T>
void complete_planes_on_host(T* h, size_t plane) {
    T* p0 = h;
    T* p1 = h + plane;
    T* p2 = h + 2 * plane;
    T* p3 = h + 3 * plane;
    T* p4 = h + 4 * plane;
    T* p5 = h + 5 * plane;
    T* p6 = h + 6 * plane;
    T* p7 = h + 7 * plane;
    T* p8 = h + 8 * plane;
    const long long n = (long long)plane;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) {
        const double ee = p0[i], em = p1[i], me = p3[i], mm = p4[i];
        p2[i] = (T)std::max(0.0, 1.0 - ee - em);  // e -> tau
        p5[i] = (T)std::max(0.0, 1.0 - me - mm);  // mu -> tau
        p6[i] = (T)std::max(0.0, 1.0 - ee - me);  // tau -> e
        p7[i] = (T)std::max(0.0, 1.0 - em - mm);  // tau -> mu
        p8[i] = (T)std::max(0.0, ee + em + me + mm - 1.0);  // tau -> tau
    }
}

}  // namespace

extern "C" {

int cp3_abi_version(void) { return CP3_ABI_VERSION; }

int cp3_bounds_checked(void) { return cp3::kChecked ? 1 : 0; }

const char* cp3_last_error(void) { return g_last_error.c_str(); }

int cp3_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int cp3_create(cp3_propagator** out, int device_id, int n_cosines, int n_energies, int precision) {
    if (!out) return fail(CP3_ERR_ARGUMENT, "cp3_create: null output pointer");
    *out = nullptr;
    if (n_cosines < 0 || n_energies < 0) return fail(CP3_ERR_ARGUMENT, "cp3_create: negative grid size");
    if (precision != CP3_PRECISION_FP64 && precision != CP3_PRECISION_MIXED)
        return fail(CP3_ERR_ARGUMENT, "cp3_create: unknown precision");
    int n_dev = 0;
    cudaError_t e = cudaGetDeviceCount(&n_dev);
    if (e != cudaSuccess || n_dev == 0) {
        cudaGetLastError();
        return fail(CP3_ERR_NO_DEVICE, "No GPU found");
    }
    if (device_id < 0 || device_id >= n_dev)
        return fail(CP3_ERR_NO_DEVICE,
                    "The requested GPU Id " + std::to_string(device_id) + " is not available.");
    DeviceGuard g(device_id);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cp3_propagator* p = new cp3_propagator();
    p->device = device_id;
    p->n_cos = n_cosines;
    p->n_en = n_energies;
    p->mixed = (precision == CP3_PRECISION_MIXED);
    p->energies.assign(n_energies, 0.0);
    p->cosines.assign(n_cosines, 0.0);
    p->maxlayers.assign(n_cosines, 0);
    if (!p->mixed) {
        p->te = 64;
        p->groups = 2;
        p->cchunk = 32;
    }
    auto bail = [&](cudaError_t err, const char* where) {
        int rc = cuda_fail(err, where);
        cp3_destroy(p);
        return rc;
    };
    if ((e = cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    p->stream = p->own_stream;
    if ((e = p->d_energy.ensure(std::max(n_energies, 1))) != cudaSuccess) return bail(e, "cudaMalloc");
    if ((e = p->d_cosine.ensure(std::max(n_cosines, 1))) != cudaSuccess) return bail(e, "cudaMalloc");
    if ((e = p->d_maxl.ensure(std::max(n_cosines, 1))) != cudaSuccess) return bail(e, "cudaMalloc");
    if ((e = p->d_result.ensure(std::max<size_t>(p->result_bytes(), 16))) != cudaSuccess)
        return bail(e, "cudaMalloc");
    {
        // cos/sin of 2*pi*j/256, j = -128..128 (Q1.30 and float, or FP64)
        std::vector<int4> tab(cp3::kPhaseTabN + 1);
        cp3::fill_phase_table(p->mixed, tab.data());
        if ((e = p->d_ptab.ensure(tab.size())) != cudaSuccess) return bail(e, "cudaMalloc");
        if ((e = cudaMemcpy(p->d_ptab.p, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return bail(e, "cudaMemcpy");
    }
    *out = p;
    return CP3_OK;
}

int cp3_destroy(cp3_propagator* p) {
    if (!p) return CP3_OK;
    DeviceGuard g(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    p->d_energy.release();
    p->d_cosine.release();
    p->d_radii.release();
    p->d_rhoye.release();
    p->d_maxl.release();
    p->d_tab.release();
    p->d_pe.release();
    p->d_len.release();
    p->d_result.release();
    p->d_ptab.release();
    p->d_flux.release();
    p->d_cbin.release();
    p->d_ebin.release();
    p->d_hist.release();
    p->d_heights.release();
    p->d_hw.release();
    p->d_lenh.release();
    if (p->h_result) cudaFreeHost(p->h_result);
    for (auto& e : p->ev)
        if (e) cudaEventDestroy(e);
    if (p->own_stream) cudaStreamDestroy(p->own_stream);
    delete p;
    return CP3_OK;
}

int cp3_set_energy_list(cp3_propagator* p, const double* list, int n) {
    if (int rc = check(p)) return rc;
    if (n != p->n_en)
        return fail(CP3_ERR_ARGUMENT,
                    "Propagator::setEnergyList. Propagator was not created for this number of energy nodes");
    if (n > 0 && !list) return fail(CP3_ERR_ARGUMENT, "setEnergyList: null list");
    for (int i = 0; i < n; i++)
        if (!(list[i] > 0.0) || !std::isfinite(list[i]))
            return fail(CP3_ERR_ARGUMENT, "setEnergyList: energies must be finite and positive");
    p->energies.assign(list, list + n);
    p->has_energy = true;
    p->energy_dirty = true;
    return CP3_OK;
}

int cp3_set_production_height(cp3_propagator* p, double height_km) {
    if (int rc = check(p)) return rc;
    if (!p->is_set_cosine) return fail(CP3_ERR_STATE, "must set cosine list before production height");
    if (!std::isfinite(height_km)) return fail(CP3_ERR_ARGUMENT, "setProductionHeight: height must be finite");
    p->height_cm = height_km * 100000.0;
    p->is_set_height = true;
    p->n_h = 0;
    return CP3_OK;
}

int cp3_set_production_heights(cp3_propagator* p, const double* heights_km, const double* weights, int n) {
    if (int rc = check(p)) return rc;
    if (!p->is_set_cosine) return fail(CP3_ERR_STATE, "must set cosine list before production height");
    if (n < 1 || n > CP3_MAX_HEIGHTS)
        return fail(CP3_ERR_ARGUMENT, "setProductionHeights: between 1 and CP3_MAX_HEIGHTS heights");
    if (!heights_km || !weights) return fail(CP3_ERR_ARGUMENT, "setProductionHeights: null list");
    double wsum = 0.0;
    for (int i = 0; i < n; i++) {
        if (!std::isfinite(heights_km[i]) || heights_km[i] < 0.0)
            return fail(CP3_ERR_ARGUMENT, "setProductionHeights: heights must be finite and >= 0");
        if (!std::isfinite(weights[i]) || weights[i] < 0.0)
            return fail(CP3_ERR_ARGUMENT, "setProductionHeights: weights must be finite and >= 0");
        wsum += weights[i];
    }
    if (!(wsum > 0.0)) return fail(CP3_ERR_ARGUMENT, "setProductionHeights: weights must not all be zero");
    if (n == 1) return cp3_set_production_height(p, heights_km[0]);
    p->heights_cm.resize(n);
    p->height_w.resize(n);
    for (int i = 0; i < n; i++) {
        p->heights_cm[i] = heights_km[i] * 100000.0;
        p->height_w[i] = weights[i] / wsum;
    }
    p->height_cm = p->heights_cm[0];
    p->n_h = n;
    p->heights_dirty = true;
    p->is_set_height = true;
    return CP3_OK;
}

int cp3_set_cosine_list(cp3_propagator* p, const double* list, int n) {
    if (int rc = check(p)) return rc;
    if (n != p->n_cos)
        return fail(CP3_ERR_ARGUMENT,
                    "Propagator::setCosineList. Propagator was not created for this number of cosine nodes");
    if (n > 0 && !list) return fail(CP3_ERR_ARGUMENT, "setCosineList: null list");
    for (int i = 0; i < n; i++)
        if (!(list[i] >= -1.0 && list[i] <= 1.0))
            return fail(CP3_ERR_ARGUMENT, "setCosineList: cosines must lie in [-1, 1]");
    p->cosines.assign(list, list + n);
    // propagator.hpp:266-268 re-sets the height through km, a round trip that
    // can move it by one ulp; kept so that path lengths match bit for bit
    if (p->is_set_height) p->height_cm = (p->height_cm / 100000.0) * 100000.0;
    set_maxlayers(p);
    p->is_set_cosine = true;
    p->cosine_dirty = true;
    return CP3_OK;
}

int cp3_set_mns_matrix(cp3_propagator* p, double t12, double t13, double t23, double dcp) {
    if (int rc = check(p)) return rc;
    if (!std::isfinite(t12) || !std::isfinite(t13) || !std::isfinite(t23) || !std::isfinite(dcp))
        return fail(CP3_ERR_ARGUMENT, "setMNSMatrix: angles must be finite");
    p->th12 = t12;
    p->th13 = t13;
    p->th23 = t23;
    p->dcp = dcp;
    p->has_mns = true;
    return CP3_OK;
}

int cp3_set_neutrino_masses(cp3_propagator* p, double dm12sq, double dm23sq) {
    if (int rc = check(p)) return rc;
    if (!std::isfinite(dm12sq) || !std::isfinite(dm23sq))
        return fail(CP3_ERR_ARGUMENT, "setNeutrinoMasses: mass splittings must be finite");
    p->dm12 = dm12sq;
    p->dm23 = dm23sq;
    p->has_masses = true;
    return CP3_OK;
}

int cp3_set_density(cp3_propagator* p, const double* radii, const double* rhos, const double* ye, int n) {
    if (int rc = check(p)) return rc;
    if (n <= 0) return fail(CP3_ERR_ARGUMENT, "setDensity : vectors must not be empty");
    if (!radii || !rhos) return fail(CP3_ERR_ARGUMENT, "setDensity : null array");
    if (n > CP3_MAX_ROWS)
        return fail(CP3_ERR_LIMIT, "setDensity : more than " + std::to_string(CP3_MAX_ROWS) + " rows");
    // propagator.hpp:127-158: one monotone order, flipped to outside-in; cosine limits
    cp3::BodyRow rows[CP3_MAX_ROWS];
    if (const char* msg = cp3::order_body(radii, rhos, ye, n, rows)) return fail(CP3_ERR_ARGUMENT, msg);
    p->radii.resize(n);
    p->rhos.resize(n);
    p->ye.resize(n);
    p->coslimit.resize(n);
    for (int i = 0; i < n; i++) {
        p->radii[i] = rows[i].radius;
        p->rhos[i] = rows[i].rho;
        p->ye[i] = rows[i].ye;
        p->coslimit[i] = rows[i].coslimit;
    }
    set_maxlayers(p);
    p->has_density = true;
    p->density_dirty = true;
    return CP3_OK;
}

int cp3_set_density_from_file(cp3_propagator* p, const char* path) {
    if (int rc = check(p)) return rc;
    if (!path) return fail(CP3_ERR_ARGUMENT, "setDensityFromFile: null path");
    std::ifstream file(path);
    if (!file) return fail(CP3_ERR_FILE, std::string("could not open density file ") + path);
    std::vector<double> r, d;
    double a, b;
    while (file >> a >> b) {
        r.push_back(a);
        d.push_back(b);
    }
    return cp3_set_density(p, r.data(), d.data(), nullptr, (int)r.size());
}

int cp3_set_stream(cp3_propagator* p, void* s) {
    if (int rc = check(p)) return rc;
    p->stream = s ? (cudaStream_t)s : p->own_stream;
    return CP3_OK;
}

int cp3_set_result_buffer(cp3_propagator* p, void* dptr, size_t bytes) {
    if (int rc = check(p)) return rc;
    if (dptr && bytes < p->result_bytes())
        return fail(CP3_ERR_ARGUMENT, "set_result_buffer: buffer smaller than 9*n_cos*n_en elements");
    p->ext_result = dptr;
    p->ext_bytes = dptr ? bytes : 0;
    p->ext_host = nullptr;
    p->completion_pending = false;
    p->results_on_host = false;
    return CP3_OK;
}

int cp3_set_host_result_buffer(cp3_propagator* p, void* host, size_t bytes) {
    if (int rc = check(p)) return rc;
    if (!host) return cp3_set_result_buffer(p, nullptr, 0);
    if (bytes < p->result_bytes())
        return fail(CP3_ERR_ARGUMENT, "set_host_result_buffer: buffer smaller than 9*n_cos*n_en elements");
    DeviceGuard g(p->device);
    // page-locked memory reports cudaMemoryTypeHost and its device alias;
    // pageable memory reports cudaMemoryTypeUnregistered
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, host);
    void* dptr = (e == cudaSuccess && at.type == cudaMemoryTypeHost) ? at.devicePointer : nullptr;
    if (!dptr) {
        cudaGetLastError();
        return fail(CP3_ERR_ARGUMENT,
                    "set_host_result_buffer: not page-locked host memory (use cudaHostAlloc or cudaHostRegister)");
    }
    p->ext_result = dptr;
    p->ext_bytes = bytes;
    p->ext_host = host;
    p->results_on_host = false;
    return CP3_OK;
}

namespace {

// prep + propagate of one calculation on the handle's stream: the nine
// planes (rates = false) or the fused rate histograms (rates = true).
int calc_async(cp3_propagator* p, int type, bool rates) {
    if (int rc = check(p)) return rc;
    if (!p->is_set_height)
        return fail(CP3_ERR_STATE, "CudaPropagatorSingle::calculateProbabilities. production height was not set");
    if (!p->has_density) return fail(CP3_ERR_STATE, "CudaPropagatorSingle::calculateProbabilities. density was not set");
    if (!p->has_mns || !p->has_masses)
        return fail(CP3_ERR_STATE,
                    "CudaPropagatorSingle::calculateProbabilities. mixing matrix or neutrino masses were not set");
    if (p->n_en > 0 && !p->has_energy)
        return fail(CP3_ERR_STATE, "CudaPropagatorSingle::calculateProbabilities. energy list was not set");
    if (type != CP3_NEUTRINO && type != CP3_ANTINEUTRINO)
        return fail(CP3_ERR_ARGUMENT, "calculateProbabilities: unknown neutrino type");
    if (rates && p->n_h > 1)
        return fail(CP3_ERR_STATE, "calculateRates: not available with a production-height distribution");
    const int mode = rates ? 1 : (p->n_h > 1 ? 2 : (p->ext_host && p->host_completion ? 3 : 0));
    if (!rates) p->results_on_host = false;
    p->completion_pending = (mode == 3);
    p->last_launches = 0;
    if (p->n_cos == 0 || p->n_en == 0) return CP3_OK;
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaGetLastError();  // a failed earlier call must not be reported by the launch checks below
    cudaError_t e;
    const int n = (int)p->radii.size();
    const int nl = n + 1;
    const int nl_pad = (nl + 1) / 2 * 2;
    // uploads of changed inputs (cudapropagator.cuh:132-159, 184-188)
    if (p->energy_dirty) {
        if ((e = cudaMemcpyAsync(p->d_energy.p, p->energies.data(), sizeof(double) * p->n_en,
                                 cudaMemcpyHostToDevice, p->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(energies)");
        p->energy_dirty = false;
    }
    if (p->cosine_dirty) {
        if ((e = cudaMemcpyAsync(p->d_cosine.p, p->cosines.data(), sizeof(double) * p->n_cos,
                                 cudaMemcpyHostToDevice, p->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(cosines)");
        p->cosine_dirty = false;
    }
    if (p->maxl_dirty) {
        if ((e = cudaMemcpyAsync(p->d_maxl.p, p->maxlayers.data(), sizeof(int) * p->n_cos, cudaMemcpyHostToDevice,
                                 p->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(maxlayers)");
        p->maxl_dirty = false;
    }
    if (p->density_dirty) {
        std::vector<double> rhoye(nl);
        rhoye[0] = 0.0;
        for (int i = 0; i < n; i++) rhoye[i + 1] = p->rhos[i] * p->ye[i];
        if ((e = p->d_radii.ensure(n)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        if ((e = p->d_rhoye.ensure(nl)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        if ((e = cudaMemcpyAsync(p->d_radii.p, p->radii.data(), sizeof(double) * n, cudaMemcpyHostToDevice,
                                 p->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(radii)");
        if ((e = cudaMemcpyAsync(p->d_rhoye.p, rhoye.data(), sizeof(double) * nl, cudaMemcpyHostToDevice,
                                 p->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync(rhoye)");
        // the staged copy must finish before `rhoye` leaves scope
        if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
        p->density_dirty = false;
    }
    // launch shape: the energy tile must leave room for the layer table
    int te = p->te, groups = p->groups, cchunk = p->cchunk;
    size_t smem = cp3::propagate_smem_bytes(p->mixed, te, nl, nl_pad, cchunk);
    const size_t smem_max = (size_t)cp3::max_dynamic_smem();
    while (smem > smem_max && te > 32) {
        te /= 2;
        groups = std::min(groups * 2, cp3::propagate_max_threads(p->mixed) / te);
        smem = cp3::propagate_smem_bytes(p->mixed, te, nl, nl_pad, cchunk);
    }
    while (smem > smem_max && cchunk > 8) {
        cchunk /= 2;
        smem = cp3::propagate_smem_bytes(p->mixed, te, nl, nl_pad, cchunk);
    }
    if (smem > smem_max) return fail(CP3_ERR_LIMIT, "density table too large for one energy tile");
    const int n_en_pad = (p->n_en + te - 1) / te * te;
    const size_t word = p->mixed ? 4 : 8;
    const size_t W = p->mixed ? cp3::kMixedWords : cp3::kFp64Words;
    if ((e = p->d_tab.ensure((size_t)n_en_pad * nl * W * word)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = p->d_pe.ensure((size_t)cp3::kPerEWords * n_en_pad * word)) != cudaSuccess)
        return cuda_fail(e, "cudaMalloc");
    if ((e = p->d_len.ensure((size_t)p->n_cos * nl_pad * 8)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if (mode == 2) {
        const int nh = p->n_h;
        if ((e = p->d_heights.ensure(nh)) != cudaSuccess || (e = p->d_hw.ensure((size_t)nh * 8)) != cudaSuccess ||
            (e = p->d_lenh.ensure((size_t)p->n_cos * nh * 8)) != cudaSuccess)
            return cuda_fail(e, "cudaMalloc");
        if (p->heights_dirty) {
            std::vector<unsigned char> wbuf((size_t)nh * 8);
            for (int i = 0; i < nh; i++) {
                if (p->mixed)
                    ((float*)wbuf.data())[i] = (float)p->height_w[i];
                else
                    ((double*)wbuf.data())[i] = p->height_w[i];
            }
            if ((e = cudaMemcpyAsync(p->d_heights.p, p->heights_cm.data(), sizeof(double) * nh,
                                     cudaMemcpyHostToDevice, p->stream)) != cudaSuccess ||
                (e = cudaMemcpyAsync(p->d_hw.p, wbuf.data(), wbuf.size(), cudaMemcpyHostToDevice, p->stream)) !=
                    cudaSuccess)
                return cuda_fail(e, "cudaMemcpyAsync(heights)");
            // the staged copy must finish before `wbuf` leaves scope
            if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
            p->heights_dirty = false;
        }
    }

    cp3::PrepArgs pa{};
    pa.pb.n_cos = p->n_cos;
    pa.pb.n_en = p->n_en;
    pa.pb.n_en_pad = n_en_pad;
    pa.pb.te = te;
    pa.pb.nl = nl;
    pa.pb.nl_pad = nl_pad;
    pa.pb.energies = p->d_energy.p;
    pa.pb.cosines = p->d_cosine.p;
    pa.pb.maxlayers = p->d_maxl.p;
    pa.pb.radii = p->d_radii.p;
    pa.pb.rhoye = p->d_rhoye.p;
    pa.pb.height_cm = p->height_cm;
    // propagator.hpp:226-248 (degeneracy break) and 191-221 (mixing matrix)
    cp3::fill_osc_params(pa.osc, p->th12, p->th13, p->th23, p->dcp, p->dm12, p->dm23, type == CP3_ANTINEUTRINO);
    pa.tab = p->d_tab.p;
    pa.pe = p->d_pe.p;
    pa.len = p->d_len.p;
    if (mode == 2) {
        pa.heights_cm = p->d_heights.p;
        pa.n_h = p->n_h;
        pa.lenh = p->d_lenh.p;
    }
    if (p->timing && (e = cudaEventRecord(p->ev[0], p->stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    if ((e = cp3::launch_prep(p->mixed, pa, p->stream)) != cudaSuccess) return cuda_fail(e, "prep kernel");
    if (p->timing && (e = cudaEventRecord(p->ev[1], p->stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");

    cp3::PropArgs ka{};
    ka.tab = p->d_tab.p;
    ka.pe = p->d_pe.p;
    ka.len = p->d_len.p;
    ka.maxl = p->d_maxl.p;
    ka.ptab = p->d_ptab.p;
    ka.out = p->result_ptr();
    ka.n_cos = p->n_cos;
    ka.n_en = p->n_en;
    ka.n_en_pad = n_en_pad;
    ka.nl = nl;
    ka.nl_pad = nl_pad;
    ka.cchunk = cchunk;
    if (rates) {
        ka.flux = p->rate_flux();
        ka.flux_mask = p->flux_mask;
        ka.cbin = p->d_cbin.p;
        ka.ebin = p->d_ebin.p;
        ka.hist = p->d_hist.p;
        ka.n_cb = p->n_cb;
        ka.n_eb = p->n_eb;
        const size_t hb = (size_t)3 * p->n_cb * p->n_eb * sizeof(double);
        if ((e = cudaMemsetAsync(p->d_hist.p, 0, hb, p->stream)) != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    if (mode == 2) {
        ka.lenh = p->d_lenh.p;
        ka.hw = p->d_hw.p;
        ka.n_h = p->n_h;
    }
    if ((e = cp3::launch_propagate(p->mixed, ka, te, groups, smem, p->stream, mode)) != cudaSuccess)
        return cuda_fail(e, "propagate kernel");
    if (p->timing && (e = cudaEventRecord(p->ev[2], p->stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    p->last_launches = 2;
    return CP3_OK;
}

}  // namespace

int cp3_calculate_probabilities_async(cp3_propagator* p, int type) { return calc_async(p, type, false); }

// ------------------------------------------------------------ event rates --
int cp3_set_rate_flux(cp3_propagator* p, const float* flux, int flavour_mask, int on_device) {
    if (int rc = check(p)) return rc;
    if (flavour_mask < 0 || flavour_mask > 7) return fail(CP3_ERR_ARGUMENT, "set_rate_flux: flavour mask must be in 0..7");
    if (flavour_mask && !flux) return fail(CP3_ERR_ARGUMENT, "set_rate_flux: null flux");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    p->ext_flux = nullptr;
    p->flux_mask = flavour_mask;
    const size_t plane = (size_t)p->n_cos * p->n_en;
    if (on_device) {
        p->ext_flux = flux;
    } else if (flavour_mask && plane) {
        cudaError_t e = p->d_flux.ensure(3 * plane);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        for (int a = 0; a < 3; a++)
            if (flavour_mask & (1 << a)) {
                e = cudaMemcpyAsync(p->d_flux.p + a * plane, flux + a * plane, plane * sizeof(float),
                                    cudaMemcpyHostToDevice, p->stream);
                if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(flux)");
            }
        if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    }
    p->has_flux = true;
    return CP3_OK;
}

int cp3_set_rate_bins(cp3_propagator* p, const int* cos_bin, const int* en_bin, int n_cos_bins, int n_en_bins) {
    if (int rc = check(p)) return rc;
    if (n_cos_bins <= 0 || n_en_bins <= 0) return fail(CP3_ERR_ARGUMENT, "set_rate_bins: bin counts must be positive");
    if ((p->n_cos && !cos_bin) || (p->n_en && !en_bin)) return fail(CP3_ERR_ARGUMENT, "set_rate_bins: null bin list");
    for (int i = 0; i < p->n_cos; i++)
        if (cos_bin[i] < -1 || cos_bin[i] >= n_cos_bins)
            return fail(CP3_ERR_ARGUMENT, "set_rate_bins: cosine bin index out of range (-1 excludes)");
    for (int i = 0; i < p->n_en; i++)
        if (en_bin[i] < -1 || en_bin[i] >= n_en_bins)
            return fail(CP3_ERR_ARGUMENT, "set_rate_bins: energy bin index out of range (-1 excludes)");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaError_t e;
    if ((e = p->d_cbin.ensure(p->n_cos)) != cudaSuccess || (e = p->d_ebin.ensure(p->n_en)) != cudaSuccess ||
        (e = p->d_hist.ensure((size_t)3 * n_cos_bins * n_en_bins)) != cudaSuccess)
        return cuda_fail(e, "cudaMalloc");
    if ((p->n_cos && (e = cudaMemcpyAsync(p->d_cbin.p, cos_bin, sizeof(int) * p->n_cos, cudaMemcpyHostToDevice,
                                          p->stream)) != cudaSuccess) ||
        (p->n_en && (e = cudaMemcpyAsync(p->d_ebin.p, en_bin, sizeof(int) * p->n_en, cudaMemcpyHostToDevice,
                                         p->stream)) != cudaSuccess) ||
        (e = cudaMemsetAsync(p->d_hist.p, 0, sizeof(double) * 3 * n_cos_bins * n_en_bins, p->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
        return cuda_fail(e, "set_rate_bins upload");
    p->n_cb = n_cos_bins;
    p->n_eb = n_en_bins;
    p->has_bins = true;
    return CP3_OK;
}

int cp3_calculate_rates_async(cp3_propagator* p, int type) {
    if (int rc = check(p)) return rc;
    if (!p->has_flux) return fail(CP3_ERR_STATE, "calculateRates: flux was not set");
    if (!p->has_bins) return fail(CP3_ERR_STATE, "calculateRates: bins were not set");
    if (p->n_cos == 0 || p->n_en == 0) {
        DeviceGuard g(p->device);
        cudaError_t e = cudaMemsetAsync(p->d_hist.p, 0, sizeof(double) * 3 * p->n_cb * p->n_eb, p->stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    return calc_async(p, type, true);
}

int cp3_calculate_rates(cp3_propagator* p, int type) {
    int rc = cp3_calculate_rates_async(p, type);
    if (rc != CP3_OK) return rc;
    return cp3_wait_for_completion(p);
}

int cp3_rates_device_ptr(cp3_propagator* p, double** dptr) {
    if (int rc = check(p)) return rc;
    if (!dptr) return fail(CP3_ERR_ARGUMENT, "null output pointer");
    if (!p->has_bins) return fail(CP3_ERR_STATE, "rates_device_ptr: bins were not set");
    *dptr = p->d_hist.p;
    return CP3_OK;
}

int cp3_get_rates(cp3_propagator* p, double* host, size_t count) {
    if (int rc = check(p)) return rc;
    if (!p->has_bins) return fail(CP3_ERR_STATE, "get_rates: bins were not set");
    const size_t n = (size_t)3 * p->n_cb * p->n_eb;
    if (!host || count < n) return fail(CP3_ERR_ARGUMENT, "get_rates: destination smaller than 3*n_cos_bins*n_en_bins");
    DeviceGuard g(p->device);
    cudaError_t e = cudaMemcpyAsync(host, p->d_hist.p, n * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(rates)");
    return CP3_OK;
}

int cp3_wait_for_completion(cp3_propagator* p) {
    if (int rc = check(p)) return rc;
    DeviceGuard g(p->device);
    cudaError_t e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (cp3::kChecked) {  // the bounds-checked build reports the calculation's failed checks here
        cp3::CheckRecord r{};
        if ((e = cp3::kernels_check_take(&r)) != cudaSuccess) return cuda_fail(e, "bounds-check record");
        if (int rc = cp3::check_status(r)) return rc;
    }
    if (p->completion_pending) {
        const size_t plane = (size_t)p->n_cos * p->n_en;
        if (p->mixed)
            complete_planes_on_host((float*)p->ext_host, plane);
        else
            complete_planes_on_host((double*)p->ext_host, plane);
        p->completion_pending = false;
    }
    return CP3_OK;
}

int cp3_set_host_completion(cp3_propagator* p, int enable) {
    if (int rc = check(p)) return rc;
    p->host_completion = enable != 0;
    return CP3_OK;
}

int cp3_calculate_probabilities(cp3_propagator* p, int type) {
    int rc = cp3_calculate_probabilities_async(p, type);
    if (rc != CP3_OK) return rc;
    return cp3_wait_for_completion(p);
}

int cp3_result_bytes(cp3_propagator* p, size_t* bytes) {
    if (int rc = check(p)) return rc;
    if (!bytes) return fail(CP3_ERR_ARGUMENT, "null output pointer");
    *bytes = p->result_bytes();
    return CP3_OK;
}

int cp3_result_device_ptr(cp3_propagator* p, void** dptr) {
    if (int rc = check(p)) return rc;
    if (!dptr) return fail(CP3_ERR_ARGUMENT, "null output pointer");
    *dptr = p->result_ptr();
    return CP3_OK;
}

int cp3_copy_results_to_host(cp3_propagator* p, void* dst, size_t bytes) {
    if (int rc = check(p)) return rc;
    if (!dst || bytes < p->result_bytes()) return fail(CP3_ERR_ARGUMENT, "copy_results_to_host: destination too small");
    if (p->result_bytes() == 0) return CP3_OK;
    DeviceGuard g(p->device);
    cudaError_t e = cudaMemcpyAsync(dst, p->result_ptr(), p->result_bytes(), cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(results)");
    return CP3_OK;
}

int cp3_get_probability(cp3_propagator* p, int ic, int ie, int t, double* out) {
    if (int rc = check(p)) return rc;
    if (!out) return fail(CP3_ERR_ARGUMENT, "null output pointer");
    if (ic >= p->n_cos || ie >= p->n_en || ic < 0 || ie < 0)
        return fail(CP3_ERR_ARGUMENT, "CudaPropagatorSingle::getProbability. Invalid indices");
    if (t < 0 || t > 8) return fail(CP3_ERR_ARGUMENT, "getProbability: ProbType out of range");
    if (p->ext_host) {
        // the kernel stored the planes straight into the caller's host buffer
        if (!p->results_on_host) {
            if (int rc = cp3_wait_for_completion(p)) return rc;
            p->results_on_host = true;
        }
        const size_t idx = (size_t)t * p->n_en * p->n_cos + (size_t)ic * p->n_en + ie;
        *out = p->mixed ? (double)((const float*)p->ext_host)[idx] : ((const double*)p->ext_host)[idx];
        return CP3_OK;
    }
    if (!p->results_on_host) {
        DeviceGuard g(p->device);
        if (!p->h_result) {
            cudaError_t e = cudaMallocHost(&p->h_result, std::max<size_t>(p->result_bytes(), 16));
            if (e != cudaSuccess) {
                p->h_result = nullptr;
                return cuda_fail(e, "cudaMallocHost");
            }
        }
        int rc = cp3_copy_results_to_host(p, p->h_result, p->result_bytes());
        if (rc != CP3_OK) return rc;
        p->results_on_host = true;
    }
    const size_t idx = (size_t)t * p->n_en * p->n_cos + (size_t)ic * p->n_en + ie;
    *out = p->mixed ? (double)((const float*)p->h_result)[idx] : ((const double*)p->h_result)[idx];
    return CP3_OK;
}

int cp3_last_launch_count(cp3_propagator* p, int* launches) {
    if (int rc = check(p)) return rc;
    if (!launches) return fail(CP3_ERR_ARGUMENT, "null output pointer");
    *launches = p->last_launches;
    return CP3_OK;
}

int cp3_set_launch_shape(cp3_propagator* p, int te, int groups, int cchunk) {
    if (int rc = check(p)) return rc;
    if ((te != 32 && te != 64 && te != 128) || groups < 1 || te * groups > cp3::propagate_max_threads(p->mixed) ||
        cchunk < 1 || cchunk > 1024)
        return fail(CP3_ERR_ARGUMENT, "set_launch_shape: unsupported launch shape");
    p->te = te;
    p->groups = groups;
    p->cchunk = cchunk;
    return CP3_OK;
}

int cp3_get_launch_shape(cp3_propagator* p, int* te, int* groups, int* cchunk) {
    if (int rc = check(p)) return rc;
    if (te) *te = p->te;
    if (groups) *groups = p->groups;
    if (cchunk) *cchunk = p->cchunk;
    return CP3_OK;
}

// Every supported (te, groups, cchunk) timed on `reps` calculations of this
// handle's grid (kernel events); the fastest shape is kept.
int cp3_autotune(cp3_propagator* p, int type, int reps, int* te_out, int* groups_out, int* cchunk_out,
                 float* best_ms) {
    if (int rc = check(p)) return rc;
    if (reps < 1) reps = 1;
    const bool was_timing = p->timing;
    if (int rc = cp3_set_kernel_timing(p, 1)) return rc;
    const int tes[3] = {32, 64, 128};
    const int chunks[4] = {8, 16, 32, 64};
    float best = 1e30f;
    int bt = p->te, bg = p->groups, bc = p->cchunk;
    int rc = CP3_OK;
    for (int te : tes)
        for (int groups = 1; rc == CP3_OK && te * groups <= cp3::propagate_max_threads(p->mixed); groups *= 2) {
            if (te * groups < 64) continue;
            for (int cc : chunks) {
                if (cc < groups) continue;
                p->te = te;
                p->groups = groups;
                p->cchunk = cc;
                if ((rc = cp3_calculate_probabilities(p, type)) == CP3_ERR_LIMIT) {
                    rc = CP3_OK;
                    continue;
                }
                if (rc) break;
                float tot = 0;
                for (int r = 0; r < reps && rc == CP3_OK; r++) {
                    float a = 0, b = 0;
                    if ((rc = cp3_calculate_probabilities(p, type)) == CP3_OK &&
                        (rc = cp3_last_kernel_ms(p, &a, &b)) == CP3_OK)
                        tot += a + b;
                }
                if (rc) break;
                if (tot / reps < best) {
                    best = tot / reps;
                    bt = te;
                    bg = groups;
                    bc = cc;
                }
            }
        }
    p->te = bt;
    p->groups = bg;
    p->cchunk = bc;
    cp3_set_kernel_timing(p, was_timing ? 1 : 0);
    if (rc) return rc;
    if (te_out) *te_out = bt;
    if (groups_out) *groups_out = bg;
    if (cchunk_out) *cchunk_out = bc;
    if (best_ms) *best_ms = best;
    return CP3_OK;
}

int cp3_get_maxlayers(cp3_propagator* p, int* out, int n) {
    if (int rc = check(p)) return rc;
    if (n != p->n_cos || (n > 0 && !out)) return fail(CP3_ERR_ARGUMENT, "get_maxlayers: n must equal n_cosines");
    std::copy(p->maxlayers.begin(), p->maxlayers.end(), out);
    return CP3_OK;
}

int cp3_set_kernel_timing(cp3_propagator* p, int enable) {
    if (int rc = check(p)) return rc;
    DeviceGuard g(p->device);
    if (enable && !p->ev[0]) {
        for (auto& e : p->ev) {
            cudaError_t err = cudaEventCreate(&e);
            if (err != cudaSuccess) return cuda_fail(err, "cudaEventCreate");
        }
    }
    p->timing = enable != 0;
    return CP3_OK;
}

int cp3_last_kernel_ms(cp3_propagator* p, float* prep_ms, float* prop_ms) {
    if (int rc = check(p)) return rc;
    if (!p->timing || p->last_launches == 0) return fail(CP3_ERR_STATE, "last_kernel_ms: no timed calculation");
    DeviceGuard g(p->device);
    cudaError_t e = cudaEventSynchronize(p->ev[2]);
    float a = 0, b = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&a, p->ev[0], p->ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b, p->ev[1], p->ev[2]);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
    if (prep_ms) *prep_ms = a;
    if (prop_ms) *prop_ms = b;
    return CP3_OK;
}

}  // extern "C"

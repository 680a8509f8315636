// cudaprob3::CudaPropagatorSingle<FLOAT_T> and cudaprob3::CudaPropagator<FLOAT_T>
// over the C ABI: drop-ins for cudapropagator.cuh:39-251 and 258-458.
//
// FLOAT_T = double runs the plain FP64 kernel and returns doubles;
// FLOAT_T = float runs the mixed kernel (double-float eigen-solve, Q1.30 fixed-point
// chain, max |dP| <= 1e-6 against FP64) and returns floats.
// Unlike the reference, each object owns its parameters (no process-global
// constant memory), so objects with different parameters may coexist.
#ifndef CUDAPROB3_GB300_CUDAPROPAGATOR_HPP
#define CUDAPROB3_GB300_CUDAPROPAGATOR_HPP

#include <algorithm>
#include <iostream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "propagator.hpp"

namespace cudaprob3 {

template <class FLOAT_T>
class CudaPropagator;

template <class FLOAT_T>
class CudaPropagatorSingle : public Propagator<FLOAT_T> {
    template <typename>
    friend class CudaPropagator;

public:
    static_assert(std::is_same<FLOAT_T, float>::value || std::is_same<FLOAT_T, double>::value,
                  "FLOAT_T must be float or double");

    /// cudapropagator.cuh:50-80
    CudaPropagatorSingle(int id, int n_cosines_, int n_energies_)
        : Propagator<FLOAT_T>(n_cosines_, n_energies_), deviceId(id) {
        detail::check(cp3_create(&h, id, n_cosines_, n_energies_,
                                 std::is_same<FLOAT_T, double>::value ? CP3_PRECISION_FP64 : CP3_PRECISION_MIXED));
    }

    /// cudapropagator.cuh:86-88
    CudaPropagatorSingle(int n_cosines, int n_energies) : CudaPropagatorSingle(0, n_cosines, n_energies) {}

    ~CudaPropagatorSingle() override { cp3_destroy(h); }

    CudaPropagatorSingle(const CudaPropagatorSingle&) = delete;
    CudaPropagatorSingle& operator=(const CudaPropagatorSingle&) = delete;
    CudaPropagatorSingle(CudaPropagatorSingle&& o) noexcept
        : Propagator<FLOAT_T>(o), h(o.h), deviceId(o.deviceId), rateBins(o.rateBins) {
        o.h = nullptr;
    }
    CudaPropagatorSingle& operator=(CudaPropagatorSingle&& o) noexcept {
        if (this != &o) {
            Propagator<FLOAT_T>::operator=(o);
            cp3_destroy(h);
            h = o.h;
            deviceId = o.deviceId;
            rateBins = o.rateBins;
            o.h = nullptr;
        }
        return *this;
    }

    void setDensity(const std::vector<FLOAT_T>& r, const std::vector<FLOAT_T>& d) override {
        Propagator<FLOAT_T>::setDensity(r, d);
        const auto rr = detail::to_double(r), dd = detail::to_double(d);
        detail::check(cp3_set_density(alive(), rr.data(), dd.data(), nullptr, (int)rr.size()));
    }
    void setDensity(const std::vector<FLOAT_T>& r, const std::vector<FLOAT_T>& d,
                    const std::vector<FLOAT_T>& y) override {
        Propagator<FLOAT_T>::setDensity(r, d, y);
        const auto rr = detail::to_double(r), dd = detail::to_double(d), yy = detail::to_double(y);
        detail::check(cp3_set_density(alive(), rr.data(), dd.data(), yy.data(), (int)rr.size()));
    }
    void setMNSMatrix(FLOAT_T t12, FLOAT_T t13, FLOAT_T t23, FLOAT_T dcp) override {
        Propagator<FLOAT_T>::setMNSMatrix(t12, t13, t23, dcp);
        detail::check(cp3_set_mns_matrix(alive(), t12, t13, t23, dcp));
    }
    void setNeutrinoMasses(FLOAT_T dm12sq, FLOAT_T dm23sq) override {
        Propagator<FLOAT_T>::setNeutrinoMasses(dm12sq, dm23sq);
        detail::check(cp3_set_neutrino_masses(alive(), dm12sq, dm23sq));
    }
    void setEnergyList(const std::vector<FLOAT_T>& list) override {
        Propagator<FLOAT_T>::setEnergyList(list);
        const auto v = detail::to_double(list);
        detail::check(cp3_set_energy_list(alive(), v.data(), (int)v.size()));
    }
    void setCosineList(const std::vector<FLOAT_T>& list) override {
        Propagator<FLOAT_T>::setCosineList(list);
        const auto v = detail::to_double(list);
        detail::check(cp3_set_cosine_list(alive(), v.data(), (int)v.size()));
    }
    void setProductionHeight(FLOAT_T heightKM) override {
        Propagator<FLOAT_T>::setProductionHeight(heightKM);
        detail::check(cp3_set_production_height(alive(), heightKM));
    }

    /// cudapropagator.cuh:162-165
    void calculateProbabilities(NeutrinoType type) override {
        calculateProbabilitiesAsync(type);
        waitForCompletion();
    }

    /// cudapropagator.cuh:168-181
    FLOAT_T getProbability(int index_cosine, int index_energy, ProbType t) override {
        double v = 0;
        detail::check(cp3_get_probability(alive(), index_cosine, index_energy, (int)t, &v));
        return (FLOAT_T)v;
    }

    /// cudapropagator.cuh:191-220 (public here: no friend access is needed)
    void calculateProbabilitiesAsync(NeutrinoType type) {
        detail::check(cp3_calculate_probabilities_async(alive(), type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO));
    }
    /// cudapropagator.cuh:223-226
    void waitForCompletion() { detail::check(cp3_wait_for_completion(alive())); }

    /// Device pointer of the 9 result planes [in*3+out][n_cosines][n_energies].
    const FLOAT_T* deviceResults() {
        void* p = nullptr;
        detail::check(cp3_result_device_ptr(alive(), &p));
        return (const FLOAT_T*)p;
    }
    /// All 9 planes copied into `out` (resized to 9 * n_cosines * n_energies).
    void getResults(std::vector<FLOAT_T>& out) {
        out.resize((size_t)9 * this->n_cosines * this->n_energies);
        detail::check(cp3_copy_results_to_host(alive(), out.data(), out.size() * sizeof(FLOAT_T)));
    }
    /// Zero-copy host results: `host` is page-locked (cudaHostAlloc or
    /// cudaHostRegister) memory of >= 9 * n_cosines * n_energies elements; the
    /// kernel stores the planes straight into it and getProbability reads it
    /// without a copy.  nullptr returns to the device buffer.
    void setHostResultBuffer(FLOAT_T* host, size_t elements) {
        detail::check(cp3_set_host_result_buffer(alive(), host, elements * sizeof(FLOAT_T)));
    }
    /// With a host result buffer: store the 2x2 flavour block only and derive
    /// the other five planes on the host cores in waitForCompletion.
    void setHostCompletion(bool enable) { detail::check(cp3_set_host_completion(alive(), enable ? 1 : 0)); }
    /// Production-height distribution (no reference counterpart): the
    /// probabilities are averaged over the heights (km) with the weights
    /// (normalised); setProductionHeight ends the distribution.
    void setProductionHeights(const std::vector<FLOAT_T>& heightsKm, const std::vector<FLOAT_T>& weights) {
        if (heightsKm.size() != weights.size())
            throw std::runtime_error("setProductionHeights: one weight per height");
        const auto h = detail::to_double(heightsKm), w = detail::to_double(weights);
        detail::check(cp3_set_production_heights(alive(), h.data(), w.data(), (int)h.size()));
        this->productionHeightKM = heightsKm.empty() ? FLOAT_T(0) : heightsKm[0];
        this->isSetProductionHeight = true;
    }
    /// Fused event rates (no reference counterpart): per-(cosine, energy)
    /// weights flux[3][n_cosines][n_energies] of the initial flavours (planes
    /// with a clear bit in flavourMask are not read), copied to the device.
    void setRateFlux(const std::vector<float>& flux, int flavourMask = 7) {
        if (flux.size() != (size_t)3 * this->n_cosines * this->n_energies)
            throw std::runtime_error("setRateFlux: flux must hold 3 * n_cosines * n_energies values");
        detail::check(cp3_set_rate_flux(alive(), flux.data(), flavourMask, 0));
    }
    /// Histogram bin of every cosine / energy node (-1 leaves it out).
    void setRateBins(const std::vector<int>& cosBin, const std::vector<int>& enBin, int nCosBins, int nEnBins) {
        if (cosBin.size() != (size_t)this->n_cosines || enBin.size() != (size_t)this->n_energies)
            throw std::runtime_error("setRateBins: one bin index per cosine and per energy node");
        detail::check(cp3_set_rate_bins(alive(), cosBin.data(), enBin.data(), nCosBins, nEnBins));
        rateBins = (size_t)3 * nCosBins * nEnBins;
    }
    /// Propagate and histogram rate_b = sum_a flux_a P(a -> b) into
    /// hist[b][cosBin][enBin] (resized to 3 * nCosBins * nEnBins).
    void calculateRates(NeutrinoType type, std::vector<double>& hist) {
        detail::check(cp3_calculate_rates(alive(), type == Antineutrino ? CP3_ANTINEUTRINO : CP3_NEUTRINO));
        hist.resize(rateBins);
        detail::check(cp3_get_rates(alive(), hist.data(), hist.size()));
    }
    cp3_propagator* handle() { return h; }

private:
    cp3_propagator* alive() {
        if (!h) throw std::runtime_error("CudaPropagatorSingle::calculateProbabilities. Object has been moved from.");
        return h;
    }
    cp3_propagator* h = nullptr;
    int deviceId;
    size_t rateBins = 0;
};

/// Multi-device propagator (cudapropagator.cuh:258-458): cosines are dealt
/// cyclically to the devices; every setter is broadcast.  Device ids may
/// repeat (several independent propagators on one GPU).
template <class FLOAT_T>
class CudaPropagator : public Propagator<FLOAT_T> {
public:
    CudaPropagator(int nc, int ne) : CudaPropagator(std::vector<int>{0}, nc, ne, true) {}

    CudaPropagator(const std::vector<int>& ids, int nc, int ne, bool failOnInvalidId = true)
        : Propagator<FLOAT_T>(nc, ne) {
        const int nDevices = cp3_device_count();
        if (nDevices == 0) throw std::runtime_error("No GPU found");
        for (int id : ids) {
            if (id >= nDevices || id < 0) {
                if (failOnInvalidId)
                    throw std::runtime_error("The requested GPU Id " + std::to_string(id) + " is not available.");
                std::cout << "invalid device id found : " << id << std::endl;
            } else {
                deviceIds.push_back(id);
            }
        }
        if (deviceIds.empty()) throw std::runtime_error("No valid device id found.");
        cosineIndices.resize(deviceIds.size());
        localCosineIndices.resize(nc);
        for (int ic = 0; ic < nc; ic++) {
            const int d = ic % (int)deviceIds.size();
            cosineIndices[d].push_back(ic);
            localCosineIndices[ic] = (int)cosineIndices[d].size() - 1;
        }
        for (size_t i = 0; i < deviceIds.size() && i < size_t(nc); i++)
            parts.emplace_back(new CudaPropagatorSingle<FLOAT_T>(deviceIds[i], (int)cosineIndices[i].size(), ne));
    }

    void setDensity(const std::vector<FLOAT_T>& r, const std::vector<FLOAT_T>& d) override {
        Propagator<FLOAT_T>::setDensity(r, d);
        for (auto& p : parts) p->setDensity(r, d);
    }
    void setDensity(const std::vector<FLOAT_T>& r, const std::vector<FLOAT_T>& d,
                    const std::vector<FLOAT_T>& y) override {
        Propagator<FLOAT_T>::setDensity(r, d, y);
        for (auto& p : parts) p->setDensity(r, d, y);
    }
    void setMNSMatrix(FLOAT_T a, FLOAT_T b, FLOAT_T c, FLOAT_T d) override {
        Propagator<FLOAT_T>::setMNSMatrix(a, b, c, d);
        for (auto& p : parts) p->setMNSMatrix(a, b, c, d);
    }
    void setNeutrinoMasses(FLOAT_T a, FLOAT_T b) override {
        Propagator<FLOAT_T>::setNeutrinoMasses(a, b);
        for (auto& p : parts) p->setNeutrinoMasses(a, b);
    }
    void setEnergyList(const std::vector<FLOAT_T>& list) override {
        Propagator<FLOAT_T>::setEnergyList(list);
        for (auto& p : parts) p->setEnergyList(list);
    }
    void setCosineList(const std::vector<FLOAT_T>& list) override {
        Propagator<FLOAT_T>::setCosineList(list);
        for (size_t i = 0; i < parts.size(); i++) {
            std::vector<FLOAT_T> mine(cosineIndices[i].size());
            std::transform(cosineIndices[i].begin(), cosineIndices[i].end(), mine.begin(),
                           [&](int ic) { return this->cosineList[ic]; });
            parts[i]->setCosineList(mine);
        }
    }
    void setProductionHeight(FLOAT_T km) override {
        Propagator<FLOAT_T>::setProductionHeight(km);
        for (auto& p : parts) p->setProductionHeight(km);
    }
    void calculateProbabilities(NeutrinoType type) override {
        for (auto& p : parts) p->calculateProbabilitiesAsync(type);
        for (auto& p : parts) p->waitForCompletion();
    }
    FLOAT_T getProbability(int index_cosine, int index_energy, ProbType t) override {
        if (index_cosine < 0 || index_cosine >= this->n_cosines)
            throw std::runtime_error("CudaPropagatorSingle::getProbability. Invalid indices");
        const int d = index_cosine % (int)deviceIds.size();
        return parts[d]->getProbability(localCosineIndices[index_cosine], index_energy, t);
    }

private:
    std::vector<int> deviceIds;
    std::vector<std::vector<int>> cosineIndices;
    std::vector<int> localCosineIndices;
    std::vector<std::unique_ptr<CudaPropagatorSingle<FLOAT_T>>> parts;
};

}  // namespace cudaprob3

#endif

// cudaprob3::Propagator<FLOAT_T>: the reference's abstract API
// (propagator.hpp:43-337) over the C ABI of libcudaprob3_gb300.so.
//
// Same member names, argument meaning and std::runtime_error messages as the
// reference, so analysis code written against CUDAProb3++ compiles unchanged.
// Validation and the physics live behind the C ABI (include/cudaprob3_gb300.h);
// this class keeps the host copies that the reference's base class keeps.
#ifndef CUDAPROB3_GB300_PROPAGATOR_HPP
#define CUDAPROB3_GB300_PROPAGATOR_HPP

#include <cstddef>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../cudaprob3_gb300.h"
#include "types.hpp"

namespace cudaprob3 {

namespace detail {
inline void check(int rc) {
    if (rc != CP3_OK) throw std::runtime_error(cp3_last_error());
}
template <class T>
std::vector<double> to_double(const std::vector<T>& v) {
    return std::vector<double>(v.begin(), v.end());
}
}  // namespace detail

template <class FLOAT_T>
class Propagator {
public:
    Propagator(int n_cosines, int n_energies) : n_cosines(n_cosines), n_energies(n_energies) {
        energyList.resize(n_energies);
        cosineList.resize(n_cosines);
    }
    virtual ~Propagator() = default;

    /// propagator.hpp:117-161
    virtual void setDensity(const std::vector<FLOAT_T>& radii_, const std::vector<FLOAT_T>& rhos_) {
        if (rhos_.size() != radii_.size()) throw std::runtime_error("setDensity : rhos.size() != radii.size()");
        if (rhos_.size() == 0) throw std::runtime_error("setDensity : vectors must not be empty");
        radii = radii_;
        rhos = rhos_;
        ye.assign(radii_.size(), FLOAT_T(0.5));
    }

    /// Extension: electron fraction per row (the reference fixes it to 0.5).
    virtual void setDensity(const std::vector<FLOAT_T>& radii_, const std::vector<FLOAT_T>& rhos_,
                            const std::vector<FLOAT_T>& ye_) {
        if (ye_.size() != radii_.size()) throw std::runtime_error("setDensity : ye.size() != radii.size()");
        Propagator::setDensity(radii_, rhos_);
        ye = ye_;
    }

    /// propagator.hpp:169-184: two columns, radius (km) and density (g/cm^3)
    virtual void setDensityFromFile(const std::string& filename) {
        std::ifstream file(filename);
        if (!file) throw std::runtime_error("could not open density file " + filename);
        std::vector<FLOAT_T> r, d;
        FLOAT_T a, b;
        while (file >> a >> b) {
            r.push_back(a);
            d.push_back(b);
        }
        setDensity(r, d);
    }

    /// propagator.hpp:191-221 (radians)
    virtual void setMNSMatrix(FLOAT_T theta12, FLOAT_T theta13, FLOAT_T theta23, FLOAT_T dCP) {
        mns[0] = theta12;
        mns[1] = theta13;
        mns[2] = theta23;
        mns[3] = dCP;
    }

    /// propagator.hpp:226-248 (eV^2)
    virtual void setNeutrinoMasses(FLOAT_T dm12sq, FLOAT_T dm23sq) {
        masses[0] = dm12sq;
        masses[1] = dm23sq;
    }

    /// propagator.hpp:252-257 (GeV)
    virtual void setEnergyList(const std::vector<FLOAT_T>& list) {
        if (list.size() != size_t(n_energies))
            throw std::runtime_error(
                "Propagator::setEnergyList. Propagator was not created for this number of energy nodes");
        energyList = list;
    }

    /// propagator.hpp:261-274
    virtual void setCosineList(const std::vector<FLOAT_T>& list) {
        if (list.size() != size_t(n_cosines))
            throw std::runtime_error(
                "Propagator::setCosineList. Propagator was not created for this number of cosine nodes");
        cosineList = list;
        isSetCosine = true;
    }

    /// propagator.hpp:279-286 (km)
    virtual void setProductionHeight(FLOAT_T heightKM) {
        if (!isSetCosine) throw std::runtime_error("must set cosine list before production height");
        productionHeightKM = heightKM;
        isSetProductionHeight = true;
    }

    /// propagator.hpp:290
    virtual void calculateProbabilities(NeutrinoType type) = 0;

    /// propagator.hpp:296
    virtual FLOAT_T getProbability(int index_cosine, int index_energy, ProbType t) = 0;

protected:
    std::vector<FLOAT_T> energyList, cosineList, radii, rhos, ye;
    FLOAT_T mns[4] = {0, 0, 0, 0};
    FLOAT_T masses[2] = {0, 0};
    FLOAT_T productionHeightKM = 0;
    bool isSetCosine = false;
    bool isSetProductionHeight = false;
    int n_cosines;
    int n_energies;
};

}  // namespace cudaprob3

#endif

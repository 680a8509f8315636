// Test infrastructure only: the host-side inputs of the reference's CUDA kernel for the
// 4096 x 4096 benchmark grid, produced by the reference's own host code.
//
// CudaPropagatorSingle::calculateProbabilitiesAsync (cudapropagator.cuh:191-220)
// fills the kernel's __constant__ data on the host before each launch:
// setMixMatrix builds the mixing matrix and its AXFAC products
// (physics.hpp:130-152), setMassDifferences the mass-difference matrix
// (180-186), and callCalculateKernelAsync's prepare_getMfast the vacuum root
// order (198-253); the device arrays hold the grid, the reordered density rows
// and the layer counts that setDensity / setMaxlayers compute
// (propagator.hpp:117-161, 301-307).  This program runs exactly that host code
// (compiled with g++ from the reference's headers where they lie, see
// oracle/Makefile) and writes, per precision and neutrino type, one file with
// those bytes, so that oracle/ref_gpu_driver.cpp can launch the reference's
// kernel on a GPU machine that has no copy of the reference's sources.
//
// Workload (the bench's headline grid): cosines uniform in [-1, 0] and
// energies log-spaced over 0.1-1000 GeV (4096 each, the example driver's grid
// builders, example/main.cpp:32-69), the 11-shell body with electron fractions
// 0.468 (core) / 0.497 (mantle) passed as rho * Ye / 0.5 (the reference's
// density is always multiplied by 0.5), nominal oscillation parameters,
// production height 22 km.  The float files get the double grid and body
// rounded to float, as a float caller would pass them.
//
// File layout (little endian): "CP3RGPU1", int32 elem, type, n_cos, n_en,
// n_rows, 0; then cos[n_cos], en[n_en], radii[n_rows], rhos[n_rows] (elem
// bytes each), int32 maxlayers[n_cos], height_cm (elem bytes), the mixing
// matrix (18 elem), AXFAC (324 elem), the mass differences (9 elem) and the
// int32 root order[3].
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// CpuPropagator<float> needs these two overloads ahead of physics.hpp (its
// unqualified fabs resolves to fabs(double) otherwise, physics.hpp:303-308).
namespace cudaprob3 { namespace physics {
inline float fabs(float x) { return std::fabs(x); }
inline double fabs(double x) { return std::fabs(x); }
} }

#include "cpupropagator.hpp"

namespace {

constexpr int kN = 4096;

std::vector<double> lin(double lo, double hi, int n) {
    std::vector<double> v(n);
    const double step = (hi - lo) / double(n - 1);
    double x = lo;
    for (int i = 0; i < n - 1; i++, x += step) v[i] = x;
    v[n - 1] = hi;
    return v;
}

std::vector<double> logsp(double lo, double hi, int n) {
    std::vector<double> v(n);
    const double a = std::log(lo), b = std::log(hi), step = (b - a) / double(n - 1);
    double x = a + step;
    v[0] = lo;
    for (int i = 1; i < n - 1; i++, x += step) v[i] = std::exp(x);
    v[n - 1] = hi;
    return v;
}

// A CpuPropagator that exposes what the CUDA propagator would upload.
template <class T>
struct Exposed : cudaprob3::CpuPropagator<T> {
    Exposed(int nc, int ne) : cudaprob3::CpuPropagator<T>(nc, ne, 1) {}
    using cudaprob3::Propagator<T>::Mix_U;
    using cudaprob3::Propagator<T>::dm;
    using cudaprob3::Propagator<T>::radii;
    using cudaprob3::Propagator<T>::rhos;
    using cudaprob3::Propagator<T>::maxlayers;
    using cudaprob3::Propagator<T>::cosineList;
    using cudaprob3::Propagator<T>::energyList;
    using cudaprob3::Propagator<T>::ProductionHeightinCentimeter;
};

template <class T>
std::vector<T> cast(const std::vector<double>& v) {
    return std::vector<T>(v.begin(), v.end());
}

template <class T>
int write_case(const std::string& path, int type) {
    const std::vector<double> cos = lin(-1.0, 0.0, kN), en = logsp(0.1, 1000.0, kN);
    const double r[12] = {0.0, 1221.5, 3480.0, 3630.0, 5701.0, 5771.0, 5971.0, 6151.0, 6346.6, 6356.0, 6368.0, 6371.0};
    const double rho[12] = {13.0, 13.0, 11.3, 5.5, 5.0, 4.4, 4.0, 3.5, 3.4, 3.0, 2.6, 1.02};
    std::vector<double> radii(r, r + 12), rhos(12);
    for (int i = 0; i < 12; i++) rhos[i] = (rho[i] * (i < 3 ? 0.468 : 0.497)) / 0.5;
    Exposed<T> p(kN, kN);
    p.setEnergyList(cast<T>(en));
    p.setCosineList(cast<T>(cos));
    p.setMNSMatrix(T(0.5837), T(0.1496), T(0.8587), T(3.86));
    p.setNeutrinoMasses(T(7.42e-5), T(2.51e-3));
    p.setDensity(cast<T>(radii), cast<T>(rhos));
    p.setProductionHeight(T(22.0));
    // calculateProbabilitiesAsync's host steps (cudapropagator.cuh:200-201)
    // and callCalculateKernelAsync's (physics.hpp:737)
    cudaprob3::physics::setMixMatrix<T>(p.Mix_U.data());
    cudaprob3::physics::setMassDifferences<T>(p.dm.data());
    cudaprob3::physics::prepare_getMfast<T>(type ? cudaprob3::Antineutrino : cudaprob3::Neutrino);
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return 1;
    const int32_t head[6] = {(int32_t)sizeof(T), type, kN, kN, (int32_t)p.radii.size(), 0};
    std::fwrite("CP3RGPU1", 1, 8, f);
    std::fwrite(head, sizeof head, 1, f);
    std::fwrite(p.cosineList.data(), sizeof(T), p.cosineList.size(), f);
    std::fwrite(p.energyList.data(), sizeof(T), p.energyList.size(), f);
    std::fwrite(p.radii.data(), sizeof(T), p.radii.size(), f);
    std::fwrite(p.rhos.data(), sizeof(T), p.rhos.size(), f);
    std::fwrite(p.maxlayers.data(), sizeof(int), p.maxlayers.size(), f);
    const T h = p.ProductionHeightinCentimeter;
    std::fwrite(&h, sizeof h, 1, f);
    std::fwrite(cudaprob3::physics::mix_data, sizeof(T), 18, f);
    std::fwrite(cudaprob3::physics::A_X_factor, sizeof(T), 324, f);
    std::fwrite(cudaprob3::physics::mass_data, sizeof(T), 9, f);
    std::fwrite(cudaprob3::physics::mass_order, sizeof(int), 3, f);
    return std::fclose(f) == 0 ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s out_dir\n", argv[0]);
        return 2;
    }
    const std::string d = argv[1];
    int rc = 0;
    rc |= write_case<double>(d + "/refgpu_f64_nu.bin", 0);
    rc |= write_case<double>(d + "/refgpu_f64_nubar.bin", 1);
    rc |= write_case<float>(d + "/refgpu_f32_nu.bin", 0);
    rc |= write_case<float>(d + "/refgpu_f32_nubar.bin", 1);
    return rc;
}

// Test-only shim: exposes the reference's own CpuPropagator<FLOAT_T>
// (cpupropagator.hpp:34-108) through a flat C ABI so that Python can call it
// to produce golden vectors.  It is compiled from the reference headers where
// they lie (see oracle/Makefile) into oracle/_ref/, which is never committed.
// Nothing in the product loads this library.
#include <cmath>
#include <string>
#include <vector>
#include <stdexcept>
#include <algorithm>
#include <fstream>
#include <array>
#include <iostream>
#include <cstring>

// CpuPropagator<float> does not compile with g++ because the unqualified fabs
// in physics.hpp:303-308 resolves to fabs(double); these two overloads, seen
// first by name lookup inside cudaprob3::physics, make it build.
namespace cudaprob3 { namespace physics {
inline float fabs(float x) { return std::fabs(x); }
inline double fabs(double x) { return std::fabs(x); }
} }

#include "cpupropagator.hpp"

static thread_local std::string g_err;

template <class T>
static int run(int nc, const T* cosv, int ne, const T* ev, int nr, const T* r, const T* rho,
               T t12, T t13, T t23, T dcp, T dm12, T dm23, T h, int anti, int threads, T* out) {
    try {
        cudaprob3::CpuPropagator<T> p(nc, ne, threads);
        p.setEnergyList(std::vector<T>(ev, ev + ne));
        p.setCosineList(std::vector<T>(cosv, cosv + nc));
        p.setMNSMatrix(t12, t13, t23, dcp);
        p.setNeutrinoMasses(dm12, dm23);
        p.setDensity(std::vector<T>(r, r + nr), std::vector<T>(rho, rho + nr));
        p.setProductionHeight(h);
        p.calculateProbabilities(anti ? cudaprob3::Antineutrino : cudaprob3::Neutrino);
        for (int ic = 0; ic < nc; ic++)
            for (int ie = 0; ie < ne; ie++)
                for (int t = 0; t < 9; t++)
                    out[(size_t(ic) * ne + ie) * 9 + t] = p.getProbability(ic, ie, cudaprob3::ProbType(t));
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
    return 0;
}

// The same with the body read by the reference's own setDensityFromFile
// (propagator.hpp:169-184) from `path`.
template <class T>
static int run_file(int nc, const T* cosv, int ne, const T* ev, const char* path, T t12, T t13, T t23, T dcp,
                    T dm12, T dm23, T h, int anti, int threads, T* out) {
    try {
        cudaprob3::CpuPropagator<T> p(nc, ne, threads);
        p.setEnergyList(std::vector<T>(ev, ev + ne));
        p.setCosineList(std::vector<T>(cosv, cosv + nc));
        p.setMNSMatrix(t12, t13, t23, dcp);
        p.setNeutrinoMasses(dm12, dm23);
        p.setDensityFromFile(std::string(path));
        p.setProductionHeight(h);
        p.calculateProbabilities(anti ? cudaprob3::Antineutrino : cudaprob3::Neutrino);
        for (int ic = 0; ic < nc; ic++)
            for (int ie = 0; ie < ne; ie++)
                for (int t = 0; t < 9; t++)
                    out[(size_t(ic) * ne + ie) * 9 + t] = p.getProbability(ic, ie, cudaprob3::ProbType(t));
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
    return 0;
}

extern "C" {
int ref_calculate_file_f64(int nc, const double* c, int ne, const double* e, const char* path, double t12,
                           double t13, double t23, double dcp, double dm12, double dm23, double h, int anti,
                           int threads, double* out) {
    return run_file<double>(nc, c, ne, e, path, t12, t13, t23, dcp, dm12, dm23, h, anti, threads, out);
}
int ref_calculate_f64(int nc, const double* c, int ne, const double* e, int nr, const double* r,
                      const double* rho, double t12, double t13, double t23, double dcp,
                      double dm12, double dm23, double h, int anti, int threads, double* out) {
    return run<double>(nc, c, ne, e, nr, r, rho, t12, t13, t23, dcp, dm12, dm23, h, anti, threads, out);
}
int ref_calculate_f32(int nc, const float* c, int ne, const float* e, int nr, const float* r,
                      const float* rho, float t12, float t13, float t23, float dcp,
                      float dm12, float dm23, float h, int anti, int threads, float* out) {
    return run<float>(nc, c, ne, e, nr, r, rho, t12, t13, t23, dcp, dm12, dm23, h, anti, threads, out);
}
const char* ref_last_error(void) { return g_err.c_str(); }
}

// Drop-in check of the C++ API: the usage of the reference's example driver
// (example/main.cpp:91-138) compiled against include/cudaprob3/ and linked to
// libcudaprob3_gb300.so.  Writes raw doubles to argv[1], per propagator: its
// cosine grid, its energy grid, then [cosine][energy][9] probabilities, for
//   CudaPropagatorSingle<double>, CudaPropagatorSingle<float>,
//   CudaPropagator<double>({0, 0}), CudaPropagator<float>({0}),
//   CudaPropagator<double>({0}) and CudaPropagator<double>({0, 0, 0}).
// The 37 cosines are dealt cyclically over 2 or 3 parts (not a multiple of
// either), so getProbability's routing to (part, local index) is checked on
// uneven parts.  The grid, body and parameters are fixed; the test compares
// with the oracle.
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <vector>

#include "cudaprob3/cudaprob3.hpp"

using namespace cudaprob3;

template <class T>
static std::vector<T> linspace(T a, T b, int n) {
    std::vector<T> v(n);
    T step = (b - a) / T(n - 1), x = a;
    for (int i = 0; i < n - 1; i++, x += step) v[i] = x;
    v[n - 1] = b;
    return v;
}

template <class T>
static std::vector<T> logspace(T a, T b, int n) {
    std::vector<T> v(n);
    T la = std::log(a), lb = std::log(b), step = (lb - la) / T(n - 1), x = la + step;
    v[0] = a;
    for (int i = 1; i < n - 1; i++, x += step) v[i] = std::exp(x);
    v[n - 1] = b;
    return v;
}

template <class T>
static void run(Propagator<T>* p, int nc, int ne, const char* density_file, std::FILE* out) {
    p->setEnergyList(logspace<T>(0.5, 100.0, ne));
    p->setCosineList(linspace<T>(-1.0, 0.0, nc));
    p->setMNSMatrix(0.5837, 0.1496, 0.8587, 3.86);
    p->setNeutrinoMasses(7.42e-5, 2.51e-3);
    p->setDensityFromFile(density_file);
    p->setProductionHeight(22.0);
    p->calculateProbabilities(cudaprob3::Neutrino);
    // the grid as this FLOAT_T sees it, then the probabilities
    const std::vector<T> e = logspace<T>(0.5, 100.0, ne), c = linspace<T>(-1.0, 0.0, nc);
    for (T x : c) { const double v = x; std::fwrite(&v, sizeof v, 1, out); }
    for (T x : e) { const double v = x; std::fwrite(&v, sizeof v, 1, out); }
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < ne; j++)
            for (int t = 0; t < 9; t++) {
                const double v = p->getProbability(i, j, ProbType(t));
                std::fwrite(&v, sizeof v, 1, out);
            }
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s out.bin density.dat\n", argv[0]);
        return 2;
    }
    const int nc = 37, ne = 45;
    std::FILE* out = std::fopen(argv[1], "wb");
    if (!out) return 3;
    try {
        std::unique_ptr<Propagator<double>> a(new CudaPropagatorSingle<double>(0, nc, ne));
        run(a.get(), nc, ne, argv[2], out);
        std::unique_ptr<Propagator<float>> b(new CudaPropagatorSingle<float>(0, nc, ne));
        run(b.get(), nc, ne, argv[2], out);
        std::unique_ptr<Propagator<double>> c(new CudaPropagator<double>(std::vector<int>{0, 0}, nc, ne));
        run(c.get(), nc, ne, argv[2], out);
        std::unique_ptr<Propagator<float>> d(new CudaPropagator<float>(std::vector<int>{0}, nc, ne));
        run(d.get(), nc, ne, argv[2], out);
        std::unique_ptr<Propagator<double>> f(new CudaPropagator<double>(std::vector<int>{0}, nc, ne));
        run(f.get(), nc, ne, argv[2], out);
        std::unique_ptr<Propagator<double>> g(new CudaPropagator<double>(std::vector<int>{0, 0, 0}, nc, ne));
        run(g.get(), nc, ne, argv[2], out);
        // the reference's ordering rule and index check throw std::runtime_error
        bool threw = false;
        try {
            CudaPropagatorSingle<double> e(0, 4, 4);
            e.setProductionHeight(22.0);
        } catch (const std::runtime_error&) {
            threw = true;
        }
        if (!threw) return 4;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    std::fclose(out);
    return 0;
}

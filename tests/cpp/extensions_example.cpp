// The C++ API beyond the reference's (production-height distributions and
// fused event rates), compiled with g++ against include/cudaprob3/ only.
//   extensions_example out.bin
// writes: the height-averaged planes [nc][ne][9] (double), then the rate
// histograms [3][4][5] (double) of a CudaPropagatorSingle<double>.
#include <cmath>
#include <cstdio>
#include <memory>
#include <vector>

#include "cudaprob3/cudaprob3.hpp"

using namespace cudaprob3;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const int nc = 21, ne = 17;
    std::FILE* out = std::fopen(argv[1], "wb");
    if (!out) return 3;
    try {
        std::vector<double> cosines(nc), energies(ne);
        for (int i = 0; i < nc; i++) cosines[i] = -1.0 + 1.5 * i / (nc - 1);
        for (int j = 0; j < ne; j++) energies[j] = 0.5 * std::pow(100.0, double(j) / (ne - 1));
        CudaPropagatorSingle<double> p(0, nc, ne);
        p.setEnergyList(energies);
        p.setCosineList(cosines);
        p.setMNSMatrix(0.5837, 0.1496, 0.8587, 3.86);
        p.setNeutrinoMasses(7.42e-5, 2.51e-3);
        p.setDensity({0.0, 1220.0, 3480.0, 5701.0, 6371.0}, {13.0, 13.0, 11.3, 5.0, 3.3});
        p.setProductionHeights({10.0, 20.0, 30.0}, {1.0, 2.0, 1.0});
        p.calculateProbabilities(Neutrino);
        for (int i = 0; i < nc; i++)
            for (int j = 0; j < ne; j++)
                for (int t = 0; t < 9; t++) {
                    const double v = p.getProbability(i, j, ProbType(t));
                    std::fwrite(&v, sizeof v, 1, out);
                }
        p.setProductionHeight(22.0);
        std::vector<float> flux(3 * nc * ne, 0.0f);
        for (int i = 0; i < nc * ne; i++) {
            flux[i] = 1.0f;               // nu_e
            flux[nc * ne + i] = 2.0f;     // nu_mu
        }
        std::vector<int> cb(nc), eb(ne);
        for (int i = 0; i < nc; i++) cb[i] = i * 4 / nc;
        for (int j = 0; j < ne; j++) eb[j] = j * 5 / ne;
        p.setRateFlux(flux, 3);
        p.setRateBins(cb, eb, 4, 5);
        std::vector<double> hist;
        p.calculateRates(Neutrino, hist);
        if (hist.size() != 3 * 4 * 5) return 4;
        std::fwrite(hist.data(), sizeof(double), hist.size(), out);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    std::fclose(out);
    return 0;
}

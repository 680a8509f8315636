// Shared definitions of the GB300 Barger propagator (host and device).
//
// Physics constants are the reference's (constants.hpp:25-41, physics.hpp:442).
// The per-layer amplitude follows Barger et al. (Phys. Rev. D 22, 2718):
// eigenvalues of 2E*H from the trigonometric cubic (Eqs. 21-22, restated from
// physics.hpp:268-341) and the propagator sum over eigenvalues (Eqs. 10-11,
// physics.hpp:346-517), written here in an eigen-basis of a real matrix:
//
//   H_f = W H_r W^dagger,  W = R23 * diag(1, 1, e^{i dcp}),
//   H_r = O diag(0, dm21, dm31) O^T - fac e0 e0^T,  O = R13 R12  (real)
//
// so that every per-layer propagator is A_l = W V_l D_l V_l^T W^dagger with a
// real orthogonal V_l and D_l = diag(1, e^{i psi1}, e^{i psi2}) (phases
// relative to the first eigenvalue; a per-layer global phase drops out of
// |amplitude|^2).  The layer chain of physics.hpp:645-677 then becomes
//
//   S_r = B^T A_M B A_0,   B = A_{M-1} ... A_1   (A_l symmetric in this basis)
//       = V_1 (Y^T D_M Y) T_0 D_0 V_0^T,  Y = T_{M-1} D_{M-1} ... T_1 D_1,
//   T_l = V_{l+1}^T V_l,
//
// which needs about half the complex 3x3 products of the reference chain.
#pragma once

#include <cmath>
#include <cstdint>

namespace cp3 {

// constants.hpp:28-40 and physics.hpp:442
constexpr double kGF = 1.52588e-4;  // 2*sqrt(2)*G_F in the reference's units
constexpr double kKm2Cm = 1.0e5;
constexpr double kREarth = 6371.0;
constexpr double kLoEfac = 2.534;
constexpr double kTwoPi = 6.283185307179586476925286766559;

constexpr int kMaxRows = 64;        // density rows accepted by set_density
constexpr int kPhaseTabN = 256;     // entries per turn of the Q1.30 cos/sin table
constexpr int kPhaseTabBytes = (kPhaseTabN + 1) * 16;  // int4 per entry
constexpr int kMixedWords = 13;     // 32-bit words per (energy, layer) mixed entry
constexpr int kFp64Words = 11;      // doubles per (energy, layer) FP64 entry
constexpr int kPerEWords = 18;      // Lambda' and Gamma' per energy (see cp3_chain.cuh)

// Oscillation parameters derived on the host from setMNSMatrix and
// setNeutrinoMasses (propagator.hpp:191-248), passed by value to kernels.
struct OscParams {
    double dm01, dm02;   // DM(0,1), DM(0,2) incl. the degeneracy break
    double d1, d2;       // DM(1,0), DM(2,0): vacuum masses relative to m1
    double u00, u01, u02;  // |U(0,j)|^2 as the reference forms them
    double o[9];         // O = R13 R12, row-major
    double hv[6];        // O diag(0, d1, d2) O^T: H00, H01, H02, H11, H12, H22
    double ca, cb0, cb1, cg;  // cubic coefficients a = fac + ca, b = cb0 + fac cb1, g = fac cg
    double s23, c23, sd, cd;
    int anti;            // 1 for antineutrinos: sign of the matter term flips
    // double-float (hi, lo) splits of the constants above, for the FP32-pipe
    // eigen-solve of the mixed prep (cp3_physics.cuh layer_eigen_df)
    float ca_f[2], cb0_f[2], cb1_f[2], cg_f[2];
    float hv_f[6][2];
    float s23_f[2], c23_f[2], sd_f[2], cd_f[2];
};

// hi = x rounded to float, lo = the rest rounded to float (a double-float split)
inline void split_df(double x, float out[2]) {
    out[0] = (float)x;
    out[1] = (float)(x - (double)out[0]);
}

// OscParams from the six parameters (mixing angles and dcp in radians,
// dm21 = m2^2 - m1^2 and dm32 = m3^2 - m2^2 in eV^2): the degeneracy break of
// propagator.hpp:226-248 and the mixing matrix of propagator.hpp:191-221.
inline void fill_osc_params(OscParams& o, double th12, double th13, double th23, double dcp, double dm21, double dm32,
                            bool anti) {
    double mv[3] = {0.0, dm21, dm21 + dm32};
    if (dm21 == 0.0) mv[0] -= 5.0e-9;
    if (dm32 == 0.0) mv[2] += 5.0e-9;
    o.dm01 = mv[0] - mv[1];
    o.dm02 = mv[0] - mv[2];
    o.d1 = -o.dm01;
    o.d2 = -o.dm02;
    const double s12 = std::sin(th12), c12 = std::cos(th12);
    const double s13 = std::sin(th13), c13 = std::cos(th13);
    o.u00 = (c12 * c13) * (c12 * c13);
    o.u01 = (s12 * c13) * (s12 * c13);
    o.u02 = s13 * s13;
    const double O[9] = {c13 * c12, c13 * s12, s13, -s12, c12, 0.0, -s13 * c12, -s13 * s12, c13};
    for (int k = 0; k < 9; k++) o.o[k] = O[k];
    const int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int k = 0; k < 6; k++) {
        const int i = ij[k][0], j = ij[k][1];
        o.hv[k] = std::fma(o.d1 * O[3 * i + 1], O[3 * j + 1], (o.d2 * O[3 * i + 2]) * O[3 * j + 2]);
    }
    o.ca = o.dm01 + o.dm02;
    o.cb0 = o.dm01 * o.dm02;
    o.cb1 = o.dm01 * (1.0 - o.u01) + o.dm02 * (1.0 - o.u02);
    o.cg = o.dm01 * o.dm02 * o.u00;
    o.s23 = std::sin(th23);
    o.c23 = std::cos(th23);
    o.sd = std::sin(dcp);
    o.cd = std::cos(dcp);
    o.anti = anti ? 1 : 0;
    split_df(o.ca, o.ca_f);
    split_df(o.cb0, o.cb0_f);
    split_df(o.cb1, o.cb1_f);
    split_df(o.cg, o.cg_f);
    for (int k = 0; k < 6; k++) split_df(o.hv[k], o.hv_f[k]);
    split_df(o.s23, o.s23_f);
    split_df(o.c23, o.c23_f);
    split_df(o.sd, o.sd_f);
    split_df(o.cd, o.cd_f);
}

// One problem for the kernels (device pointers).
struct Problem {
    int n_cos, n_en;
    int n_en_pad;        // energies padded to the energy tile
    int te;              // energies per tile (table tiling and block.x)
    int nl;              // layers: 1 (vacuum) + density rows
    int nl_pad;          // row stride of the per-cosine tables
    const double* energies;  // [n_en]
    const double* cosines;   // [n_cos]
    const int* maxlayers;    // [n_cos]
    const double* radii;     // [nl-1] descending (outermost first)
    const double* rhoye;     // [nl] layer 0 = 0 (vacuum), layer l = rho*Ye of row l-1
    double height_cm;
};

}  // namespace cp3

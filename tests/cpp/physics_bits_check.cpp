// Host build of the bit-level helpers and the eigen-solve of cp3_physics.cuh
// (the same source the kernels use), checked against the conversions and
// divisions they replace.  Prints "bad <count>" and exits non-zero on any
// mismatch.
#define CP3_HD inline
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "cp3_physics.cuh"

using namespace cp3;

static long bad = 0;

static void check_q30(double x) {
    const long long want = std::llrint(x * 1073741824.0);  // round half to even
    if (q30_rn(x) != (int)want && bad++ < 5) std::printf("q30_rn(%a) = %d, want %lld\n", x, q30_rn(x), want);
}

static void check_f32(double x) {
    float want = (float)x;
    if (std::fabs(x) < 1.1754943508222875e-38) want = std::copysign(0.0f, (float)x);  // flushed below FLT_MIN
    const float got = f32_rn(x);
    if (std::memcmp(&want, &got, 4) != 0 && bad++ < 5) std::printf("f32_rn(%a) = %a, want %a\n", x, (double)got, (double)want);
    const float f = (float)x;
    const double back = f64_of(f);
    const double wantd = (std::fabs(f) < 1.17549435e-38f) ? std::copysign(0.0, (double)f) : (double)f;
    if ((std::memcmp(&back, &wantd, 8) != 0) && bad++ < 5) std::printf("f64_of(%a) = %a\n", (double)f, back);
}

int main(int argc, char** argv) {
    const long n = (argc > 1) ? std::atol(argv[1]) : 2000000;
    std::mt19937_64 g(1);
    std::uniform_real_distribution<double> u(-2.0, 2.0), cm(0.0, 1.3e9);
    for (long i = 0; i < n; i++) {
        const double x = u(g);
        if (x > -2.0 && x < 2.0) check_q30(x);
        check_f32(std::ldexp(x, (int)(g() % 80) - 40));
        const double c = cm(g);
        if (km_of_cm(c) != c / 1.0e5 && bad++ < 5) std::printf("km_of_cm(%a)\n", c);
        const double a = std::ldexp(u(g), (int)(g() % 20) - 10), b = std::ldexp(u(g), (int)(g() % 20) - 10);
        if (b != 0.0 && std::fabs(div_nr(a, b) - a / b) > 2.3e-16 * std::fabs(a / b) && bad++ < 5)
            std::printf("div_nr(%a, %a)\n", a, b);
        const double y = u(g), z = u(g);
        if (less_than(y, z) != (y < z) && bad++ < 5) std::printf("less_than(%a, %a)\n", y, z);
        if ((abs_key(y) >= abs_key(z)) != (std::fabs(y) >= std::fabs(z)) && bad++ < 5) std::printf("abs_key(%a)\n", y);
    }
    // ties of the Q1.30 rounding and halfway points between floats
    for (long k = -3000; k < 3000; k++) {
        check_q30((k + 0.5) / 1073741824.0);
        check_q30(std::ldexp((double)k + 0.5, -40));
        const double t = std::ldexp(1.0 + (2 * k + 1) * std::ldexp(1.0, -24), 3);
        check_f32(t);
        check_f32(-t);
    }
    const double edge[] = {0.0, -0.0, 1.0, -1.0, 1.9999999999, 1e-300, 1e-40, 3.4028235e38, 3.4028236e38, 1e39, -1e39};
    for (double x : edge) {
        if (std::fabs(x) < 2) check_q30(x);
        check_f32(x);
    }
    if (!std::isnan(f32_rn(NAN)) || !std::isnan(f64_of(NAN))) bad++;
    // eigen-solve: orthonormal, right-handed, eigen-pairs of 2E*H_r
    OscParams o{};
    fill_osc_params(o, 0.5837, 0.1496, 0.8587, 3.86, 7.42e-5, 2.51e-3, false);
    for (int k = 0; k < 2000; k++) {
        const double E = std::exp(std::log(0.1) + (std::log(1000.0) - std::log(0.1)) * (k % 200) / 199.0);
        const double rhoye = (k / 200) * 1.4;
        double m[3], V[9];
        layer_eigen(o, E, rhoye, m, V);
        const double fac = -(kGF * E * rhoye);
        double H[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                H[3 * i + j] = o.d1 * o.o[3 * i + 1] * o.o[3 * j + 1] + o.d2 * o.o[3 * i + 2] * o.o[3 * j + 2];
        H[0] -= fac;
        double worst = 0.0;
        for (int c = 0; c < 3; c++) {
            for (int i = 0; i < 3; i++) {
                double hv = 0.0;
                for (int j = 0; j < 3; j++) hv += H[3 * i + j] * V[3 * j + c];
                worst = std::fmax(worst, std::fabs(hv - m[c] * V[3 * i + c]));
            }
            for (int d = 0; d < 3; d++) {
                double dot = 0.0;
                for (int i = 0; i < 3; i++) dot += V[3 * i + c] * V[3 * i + d];
                worst = std::fmax(worst, std::fabs(dot - (c == d ? 1.0 : 0.0)) * 1e-2);
            }
        }
        const double det = V[0] * (V[4] * V[8] - V[5] * V[7]) - V[1] * (V[3] * V[8] - V[5] * V[6]) +
                           V[2] * (V[3] * V[7] - V[4] * V[6]);
        if ((worst > 1e-15 || std::fabs(det - 1.0) > 1e-13) && bad++ < 5)
            std::printf("layer_eigen E=%g rhoye=%g residual %g det %g\n", E, rhoye, worst, det);
    }
    // random parameters, including exact degeneracies (dm21 = 0 or dm32 = 0:
    // the 5e-9 eV^2 break), inverted ordering and vacuum layers
    std::uniform_real_distribution<double> ang(0.0, 1.5707963), ph(0.0, 6.2831853), lg(0.0, 1.0);
    double worst_res = 0.0, worst_orth = 0.0;
    for (int k = 0; k < 200000; k++) {
        const double dm21 = (k % 7 == 0) ? 0.0 : 7.4e-5 * (0.5 + lg(g));
        const double dm32 = (k % 11 == 0) ? 0.0 : ((k & 1) ? -1.0 : 1.0) * 2.5e-3 * (0.5 + lg(g));
        OscParams q{};
        fill_osc_params(q, ang(g), ang(g), ang(g), ph(g), dm21, dm32, (k & 2) != 0);
        const double E = std::exp(std::log(0.05) + lg(g) * (std::log(2000.0) - std::log(0.05)));
        const double rhoye = (k % 5 == 0) ? 0.0 : 7.0 * lg(g);
        double m[3], V[9];
        layer_eigen(q, E, rhoye, m, V);
        const double fac = q.anti ? kGF * E * rhoye : -(kGF * E * rhoye);
        double H[9], hn = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                H[3 * i + j] = q.d1 * q.o[3 * i + 1] * q.o[3 * j + 1] + q.d2 * q.o[3 * i + 2] * q.o[3 * j + 2];
                if (i == 0 && j == 0) H[0] -= fac;
                hn = std::fmax(hn, std::fabs(H[3 * i + j]));
            }
        for (int c = 0; c < 3; c++) {
            for (int i = 0; i < 3; i++) {
                double hv = 0.0;
                for (int j = 0; j < 3; j++) hv += H[3 * i + j] * V[3 * j + c];
                worst_res = std::fmax(worst_res, std::fabs(hv - m[c] * V[3 * i + c]) / hn);
            }
            for (int d = 0; d < 3; d++) {
                double dot = 0.0;
                for (int i = 0; i < 3; i++) dot += V[3 * i + c] * V[3 * i + d];
                worst_orth = std::fmax(worst_orth, std::fabs(dot - (c == d ? 1.0 : 0.0)));
            }
        }
        const double det = V[0] * (V[4] * V[8] - V[5] * V[7]) - V[1] * (V[3] * V[8] - V[5] * V[6]) +
                           V[2] * (V[3] * V[7] - V[4] * V[6]);
        if (std::fabs(det - 1.0) > 1e-12 && bad++ < 5) std::printf("det %g at case %d\n", det, k);
    }
    std::printf("random cases: residual/|H| %.3g, |V^T V - I| %.3g\n", worst_res, worst_orth);
    if (worst_res > 1e-11 || worst_orth > 1e-14) bad++;

    // double-float arithmetic (cp3_df.cuh) against FP64 on double-float inputs
    {
        double w_add = 0, w_mul = 0, w_div = 0, w_sqrt = 0;
        for (int k = 0; k < 200000; k++) {
            const double x = std::ldexp(u(g), (int)(g() % 40) - 20), y = std::ldexp(u(g), (int)(g() % 40) - 20);
            const DF a = df_from_double(x), b = df_from_double(y);
            const double xa = df_to_double(a), yb = df_to_double(b);
            const double s = xa + yb, p = xa * yb, q = xa / yb;
            if (s != 0.0) w_add = std::fmax(w_add, std::fabs(df_to_double(df_add(a, b)) - s) / std::fabs(s));
            w_mul = std::fmax(w_mul, std::fabs(df_to_double(df_mul(a, b)) - p) / std::fabs(p));
            w_div = std::fmax(w_div, std::fabs(df_to_double(df_div(a, b)) - q) / std::fabs(q));
            const double r = std::sqrt(std::fabs(xa));
            w_sqrt = std::fmax(w_sqrt, std::fabs(df_to_double(df_sqrt(df_abs(a))) - r) / r);
        }
        std::printf("double-float vs FP64: add %.3g, mul %.3g, div %.3g, sqrt %.3g (relative)\n", w_add, w_mul, w_div,
                    w_sqrt);
        // the arithmetic's bounds are a few u^2 = 2^-48 = 3.6e-15
        if (w_add > 2e-14 || w_mul > 2e-14 || w_div > 4e-14 || w_sqrt > 4e-14) bad++;
    }
    // the double-float eigen-solve of the mixed prep against the FP64 one.
    // Where no splitting is zero the two agree to the double-float precision;
    // with dm21 = 0 or dm32 = 0 the degeneracy break leaves two eigenvalues
    // 5e-9 eV^2 apart, the deflation's discriminant cancels by ~1e9, and the
    // pair's split (and its eigenvectors within their plane) is resolved to
    // ~1e-5 instead of ~1e-7 relative: those cases are held to the
    // eigen-equation and orthonormality instead
    {
        std::mt19937_64 g2(7);
        double w_m = 0, w_v = 0, w_orth = 0, w_det = 0, w_res = 0;
        for (int k = 0; k < 200000; k++) {
            const bool degenerate = (k % 7 == 0) || (k % 11 == 0);
            const double dm21 = (k % 7 == 0) ? 0.0 : 7.4e-5 * (0.5 + lg(g2));
            const double dm32 = (k % 11 == 0) ? 0.0 : ((k & 1) ? -1.0 : 1.0) * 2.5e-3 * (0.5 + lg(g2));
            const double t12 = ang(g2), t13 = ang(g2), t23 = ang(g2), dcp = ph(g2);
            OscParams q{};
            fill_osc_params(q, t12, t13, t23, dcp, dm21, dm32, (k & 2) != 0);
            const double E = std::exp(std::log(0.05) + lg(g2) * (std::log(2000.0) - std::log(0.05)));
            const double rhoye = (k % 5 == 0) ? 0.0 : 7.0 * lg(g2);
            double m[3], V[9];
            layer_eigen(q, E, rhoye, m, V);
            DF md[3], Vd[9];
            layer_eigen_df(q, df_from_double(E), df_from_double(rhoye), md, Vd);
            double Vv[9], mv[3];
            for (int i = 0; i < 9; i++) Vv[i] = df_to_double(Vd[i]);
            for (int c = 0; c < 3; c++) mv[c] = df_to_double(md[c]);
            const double fac = q.anti ? kGF * E * rhoye : -(kGF * E * rhoye);
            double H[9], hn = 0.0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    H[3 * i + j] = q.d1 * q.o[3 * i + 1] * q.o[3 * j + 1] + q.d2 * q.o[3 * i + 2] * q.o[3 * j + 2];
                    if (i == 0 && j == 0) H[0] -= fac;
                    hn = std::fmax(hn, std::fabs(H[3 * i + j]));
                }
            for (int c = 0; c < 3; c++)
                for (int i = 0; i < 3; i++) {
                    double hv = 0.0;
                    for (int j = 0; j < 3; j++) hv += H[3 * i + j] * Vv[3 * j + c];
                    w_res = std::fmax(w_res, std::fabs(hv - mv[c] * Vv[3 * i + c]) / hn);
                }
            if (!degenerate) {
                const double scale = std::fmax(std::fabs(m[0]), std::fmax(std::fabs(m[1]), std::fabs(m[2])));
                for (int c = 0; c < 3; c++) w_m = std::fmax(w_m, std::fabs(mv[c] - m[c]) / scale);
                for (int i = 0; i < 9; i++) w_v = std::fmax(w_v, std::fabs(Vv[i] - V[i]));
            }
            for (int c = 0; c < 3; c++)
                for (int d = 0; d < 3; d++) {
                    double dot = 0.0;
                    for (int i = 0; i < 3; i++) dot += Vv[3 * i + c] * Vv[3 * i + d];
                    w_orth = std::fmax(w_orth, std::fabs(dot - (c == d ? 1.0 : 0.0)));
                }
            const double det = Vv[0] * (Vv[4] * Vv[8] - Vv[5] * Vv[7]) - Vv[1] * (Vv[3] * Vv[8] - Vv[5] * Vv[6]) +
                               Vv[2] * (Vv[3] * Vv[7] - Vv[4] * Vv[6]);
            w_det = std::fmax(w_det, std::fabs(det - 1.0));
        }
        std::printf("double-float eigen-solve vs FP64 (no zero splitting): eigenvalues %.3g (of the largest), "
                    "eigenvectors %.3g; all cases: residual/|H| %.3g, |V^T V - I| %.3g, |det - 1| %.3g\n",
                    w_m, w_v, w_res, w_orth, w_det);
        // (bounds: the mixed tables are Q1.30, resolution 9.3e-10)
        if (w_m > 1e-12 || w_v > 1e-9 || w_res > 1e-9 || w_orth > 1e-10 || w_det > 1e-10) bad++;
    }
    std::printf("bad %ld\n", bad);
    return bad != 0;
}

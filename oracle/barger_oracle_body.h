/*
 * Oracle body: CPU restatement of CUDAProb3++'s CpuPropagator<FLOAT_T> path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle used by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py.  The
 * product (cudaprob3_gb300) never links, imports or calls it.
 *
 * Included twice by barger_oracle.c, once with REAL=double (SFX=_f64) and once
 * with REAL=float (SFX=_f32).  Every step follows the reference's evaluation
 * order so that the double instantiation reproduces CpuPropagator<double>
 * to the last bit on the same compiler flags (-ffp-contract=off).  The float
 * instantiation mirrors CpuPropagator<float>, where the reference calls the
 * double-precision libm routines (sqrt, acos, cos, sin) and promotes the
 * double literals 2.0, 3.0, 9.0, 27.0 and M_PI, so a part of its arithmetic
 * is double even in the float build.
 *
 * References (paths inside the reference project):
 *   propagator.hpp:117-161  setDensity (validation, flip, cosine limits)
 *   propagator.hpp:191-221  setMNSMatrix
 *   propagator.hpp:226-248  setNeutrinoMasses (degeneracy break)
 *   propagator.hpp:279-286  setProductionHeight
 *   propagator.hpp:301-307  setMaxlayers
 *   physics.hpp:130-152     setMixMatrix (AXFAC table)
 *   physics.hpp:198-253     prepare_getMfast (vacuum root order)
 *   physics.hpp:268-341     getMfast (Cardano matter eigenvalues)
 *   physics.hpp:346-431     get_product (Barger Eq. 11 projectors)
 *   physics.hpp:434-517     getA (phases, X sum, flavour rotation)
 *   physics.hpp:536-580     getDensityOfLayer / getTraversedDistanceOfLayer
 *   physics.hpp:583-702     calculate (pair loop, layer chain, writeback)
 *   math.hpp:50-64          multiply_complex_matrix (C += A*B)
 *   constants.hpp:25-41     physical constants
 */

typedef struct { REAL re, im; } CAT(cplx, SFX);
#define CPLX CAT(cplx, SFX)

/* constants.hpp:28-40, each evaluated in REAL like the reference's constexpr. */
#define K_GF      ((REAL)1.52588e-4)
#define K_KM2CM   ((REAL)1.0e5)
#define K_REARTH  ((REAL)6371.0)
#define K_DENSCONV ((REAL)0.5)

typedef struct {
    CPLX U[9];           /* Mix_U, row-major U(i,j) */
    REAL dm[9];          /* DM(i,j) */
    REAL axfac[81 * 4];  /* AXFAC(n,m,i,j,e) */
    int order[3];        /* mass_order */
} CAT(osc_state, SFX);
#define OSC CAT(osc_state, SFX)

#define U_(i, j) (st->U[(i) * 3 + (j)])
#define DM_(i, j) (st->dm[(i) * 3 + (j)])
#define AX_(n, m, i, j, e) (st->axfac[(n) * 108 + (m) * 36 + (i) * 12 + (j) * 4 + (e)])

/* propagator.hpp:191-221 */
static void CAT(set_mns, SFX)(OSC* st, REAL th12, REAL th13, REAL th23, REAL dcp) {
    const REAL s12 = sin(th12), s13 = sin(th13), s23 = sin(th23);
    const REAL c12 = cos(th12), c13 = cos(th13), c23 = cos(th23);
    const REAL sd = sin(dcp), cd = cos(dcp);
    U_(0, 0).re = c12 * c13;                    U_(0, 0).im = 0.0;
    U_(0, 1).re = s12 * c13;                    U_(0, 1).im = 0.0;
    U_(0, 2).re = s13 * cd;                     U_(0, 2).im = -s13 * sd;
    U_(1, 0).re = -s12 * c23 - c12 * s23 * s13 * cd;
    U_(1, 0).im = -c12 * s23 * s13 * sd;
    U_(1, 1).re = c12 * c23 - s12 * s23 * s13 * cd;
    U_(1, 1).im = -s12 * s23 * s13 * sd;
    U_(1, 2).re = s23 * c13;                    U_(1, 2).im = 0.0;
    U_(2, 0).re = s12 * s23 - c12 * c23 * s13 * cd;
    U_(2, 0).im = -c12 * c23 * s13 * sd;
    U_(2, 1).re = -c12 * s23 - s12 * c23 * s13 * cd;
    U_(2, 1).im = -s12 * c23 * s13 * sd;
    U_(2, 2).re = c23 * c13;                    U_(2, 2).im = 0.0;
}

/* propagator.hpp:226-248 */
static void CAT(set_masses, SFX)(OSC* st, REAL dm12sq, REAL dm23sq) {
    REAL mv[3];
    mv[0] = 0.0;
    mv[1] = dm12sq;
    mv[2] = dm12sq + dm23sq;
    const REAL delta = 5.0e-9;
    if (dm12sq == 0.0) mv[0] -= delta;
    if (dm23sq == 0.0) mv[2] += delta;
    DM_(0, 0) = 0.0; DM_(1, 1) = 0.0; DM_(2, 2) = 0.0;
    DM_(0, 1) = mv[0] - mv[1]; DM_(1, 0) = -DM_(0, 1);
    DM_(0, 2) = mv[0] - mv[2]; DM_(2, 0) = -DM_(0, 2);
    DM_(1, 2) = mv[1] - mv[2]; DM_(2, 1) = -DM_(1, 2);
}

/* physics.hpp:130-152: products U(n,i) * conj(U(m,j)) split in four parts. */
static void CAT(build_axfac, SFX)(OSC* st) {
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const CPLX a = U_(n, i), b = U_(m, j);
                    AX_(n, m, i, j, 0) = a.re * b.re + a.im * b.im;
                    AX_(n, m, i, j, 1) = a.re * b.im - a.im * b.re;
                    AX_(n, m, i, j, 2) = a.im * b.im + a.re * b.re;
                    AX_(n, m, i, j, 3) = a.im * b.re - a.re * b.im;
                }
}

/* physics.hpp:198-253: solve the vacuum cubic the same way as the matter
 * cubic and map each vacuum mass DM(i,0) to the closest root. */
static void CAT(vacuum_order, SFX)(OSC* st) {
    REAL alphaV, betaV, gammaV, argV, tmpV, t0, t1, t2;
    REAL mv[3];
    alphaV = DM_(0, 1) + DM_(0, 2);
    betaV = DM_(0, 1) * DM_(0, 2);
    gammaV = 0.0;
    tmpV = alphaV * alphaV - 3.0 * betaV;
    argV = (2.0 * alphaV * alphaV * alphaV - 9.0 * alphaV * betaV + 27.0 * gammaV) /
           (2.0 * sqrt(tmpV * tmpV * tmpV));
    if (fabs(argV) > 1.0) argV = argV / fabs(argV);
    t0 = acos(argV) / 3.0;
    t1 = t0 - (2.0 * M_PI / 3.0);
    t2 = t0 + (2.0 * M_PI / 3.0);
    mv[0] = mv[1] = mv[2] = -(2.0 / 3.0) * sqrt(tmpV);
    mv[0] *= cos(t0); mv[1] *= cos(t1); mv[2] *= cos(t2);
    tmpV = DM_(0, 0) - alphaV / 3.0;
    mv[0] += tmpV; mv[1] += tmpV; mv[2] += tmpV;
    for (int i = 0; i < 3; i++) {
        tmpV = fabs(DM_(i, 0) - mv[0]);
        int k = 0;
        for (int j = 1; j < 3; j++) {
            REAL t = fabs(DM_(i, 0) - mv[j]);
            if (t < tmpV) { k = j; tmpV = t; }
        }
        st->order[i] = k;
    }
}

/* physics.hpp:268-341: matter eigenvalues (Barger Eqs. 21-22). */
static void CAT(matter_masses, SFX)(const OSC* st, REAL E, REAL rho, int anti,
                                    REAL dMM[3][3], REAL dMV[3][3]) {
    REAL mU[3], mm[3];
    const REAL fac = anti ? K_GF * E * rho : -K_GF * E * rho;
    const REAL alpha = fac + DM_(0, 1) + DM_(0, 2);
    const REAL beta = DM_(0, 1) * DM_(0, 2) +
        fac * (DM_(0, 1) * (1.0 - U_(0, 1).re * U_(0, 1).re - U_(0, 1).im * U_(0, 1).im) +
               DM_(0, 2) * (1.0 - U_(0, 2).re * U_(0, 2).re - U_(0, 2).im * U_(0, 2).im));
    const REAL gamma = fac * DM_(0, 1) * DM_(0, 2) * (U_(0, 0).re * U_(0, 0).re + U_(0, 0).im * U_(0, 0).im);
    const REAL tmp = alpha * alpha - 3.0 * beta < 0 ? 0 : alpha * alpha - 3.0 * beta;
    const REAL argtmp = (2.0 * alpha * alpha * alpha - 9.0 * alpha * beta + 27.0 * gamma) /
                        (2.0 * sqrt(tmp * tmp * tmp));
    REAL arg;
    if (fabs(argtmp) > 1.0) arg = argtmp / fabs(argtmp); else arg = argtmp;
    const REAL th0 = acos(arg) / 3.0;
    const REAL th1 = th0 - (2.0 * M_PI / 3.0);
    const REAL th2 = th0 + (2.0 * M_PI / 3.0);
    mU[0] = -(2.0 / 3.0) * sqrt(tmp);
    mU[1] = -(2.0 / 3.0) * sqrt(tmp);
    mU[2] = -(2.0 / 3.0) * sqrt(tmp);
    mU[0] *= cos(th0); mU[1] *= cos(th1); mU[2] *= cos(th2);
    const REAL tmp2 = DM_(0, 0) - alpha / 3.0;
    mU[0] += tmp2; mU[1] += tmp2; mU[2] += tmp2;
    for (int i = 0; i < 3; i++) mm[i] = mU[st->order[i]];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            dMM[i][j] = mm[i] - mm[j];
            dMV[i][j] = mm[i] - DM_(j, 0);
        }
}

/* physics.hpp:346-431: projector numerators (2EH - M_a)(2EH - M_b) / gaps. */
static void CAT(projectors, SFX)(const OSC* st, REAL E, REAL rho, int anti,
                                 REAL dMV[3][3], REAL dMM[3][3], CPLX prod[3][3][3]) {
    CPLX t[3][3][3];
    const REAL fac = anti ? K_GF * E * rho : -K_GF * E * rho;
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++) {
            const REAL re = -fac * (U_(0, n).re * U_(0, m).re + U_(0, n).im * U_(0, m).im);
            const REAL im = -fac * (U_(0, n).re * U_(0, m).im - U_(0, n).im * U_(0, m).re);
            for (int j = 0; j < 3; j++) { t[n][m][j].re = re; t[n][m][j].im = im; }
        }
    for (int j = 0; j < 3; j++) {
        t[0][0][j].re -= dMV[j][0];
        t[1][1][j].re -= dMV[j][1];
        t[2][2][j].re -= dMV[j][2];
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) { prod[i][j][k].re = 0; prod[i][j][k].im = 0; }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            for (int k = 0; k < 3; k++) {
                prod[i][j][0].re += t[i][k][1].re * t[k][j][2].re - t[i][k][1].im * t[k][j][2].im;
                prod[i][j][0].im += t[i][k][1].re * t[k][j][2].im + t[i][k][1].im * t[k][j][2].re;
                prod[i][j][1].re += t[i][k][2].re * t[k][j][0].re - t[i][k][2].im * t[k][j][0].im;
                prod[i][j][1].im += t[i][k][2].re * t[k][j][0].im + t[i][k][2].im * t[k][j][0].re;
                prod[i][j][2].re += t[i][k][0].re * t[k][j][1].re - t[i][k][0].im * t[k][j][1].im;
                prod[i][j][2].im += t[i][k][0].re * t[k][j][1].im + t[i][k][0].im * t[k][j][1].re;
            }
            prod[i][j][0].re /= (dMM[0][1] * dMM[0][2]);
            prod[i][j][0].im /= (dMM[0][1] * dMM[0][2]);
            prod[i][j][1].re /= (dMM[1][2] * dMM[1][0]);
            prod[i][j][1].im /= (dMM[1][2] * dMM[1][0]);
            prod[i][j][2].re /= (dMM[2][0] * dMM[2][1]);
            prod[i][j][2].im /= (dMM[2][0] * dMM[2][1]);
        }
}

/* physics.hpp:434-517 (phase_offset == 0 always on this path) and
 * physics.hpp:522-531: amplitude of one constant-density segment. */
static void CAT(layer_amplitude, SFX)(const OSC* st, int anti, REAL E, REAL rho, REAL L,
                                      CPLX A[3][3]) {
    REAL dMM[3][3], dMV[3][3];
    CPLX prod[3][3][3], X[3][3];
    const REAL LoEfac = 2.534;
    CAT(matter_masses, SFX)(st, E, rho, anti, dMM, dMV);
    CAT(projectors, SFX)(st, E, rho, anti, dMV, dMM, prod);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { X[i][j].re = 0; X[i][j].im = 0; }
    for (int k = 0; k < 3; k++) {
        const REAL arg = -LoEfac * dMV[k][0] * L / E;
        const REAL s = sin(arg);
        const REAL c = cos(arg);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                X[i][j].re += c * prod[i][j][k].re - s * prod[i][j][k].im;
                X[i][j].im += c * prod[i][j][k].im + s * prod[i][j][k].re;
            }
    }
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++) { A[n][m].re = 0; A[n][m].im = 0; }
    for (int n = 0; n < 3; n++)
        for (int m = 0; m < 3; m++)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    A[n][m].re += AX_(n, m, i, j, 0) * X[i][j].re + AX_(n, m, i, j, 1) * X[i][j].im;
                    A[n][m].im += AX_(n, m, i, j, 2) * X[i][j].im + AX_(n, m, i, j, 3) * X[i][j].re;
                }
}

/* math.hpp:50-64: C += A * B. */
static void CAT(cmat_mul_acc, SFX)(CPLX A[3][3], CPLX B[3][3], CPLX C[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                C[i][j].re += A[i][k].re * B[k][j].re - A[i][k].im * B[k][j].im;
                C[i][j].im += A[i][k].im * B[k][j].re + A[i][k].re * B[k][j].im;
            }
}

static void CAT(cmat_zero, SFX)(CPLX A[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { A[i][j].re = 0; A[i][j].im = 0; }
}

static void CAT(cmat_copy, SFX)(CPLX A[3][3], CPLX B[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B[i][j] = A[i][j];
}

/* physics.hpp:555-580, with the radii already in descending order. */
static REAL CAT(layer_distance, SFX)(const REAL* radii, int layer, int maxl, REAL path,
                                     REAL earth, REAL c) {
    if (c >= 0) return path;
    if (layer == 0) return path - earth;
    const int i = (layer >= maxl) ? (-layer - 1 + 2 * maxl) : (layer - 1);
    const REAL R = K_REARTH;
    const REAL cross_this = 2.0 * sqrt(radii[i] * radii[i] - R * R * (1 - c * c));
    if (i < maxl - 1) {
        const REAL cross_next = 2.0 * sqrt(radii[i + 1] * radii[i + 1] - R * ((REAL)K_REARTH) * (1 - c * c));
        return 0.5 * (cross_this - cross_next) * K_KM2CM;
    }
    return cross_this * K_KM2CM;
}

/* physics.hpp:538-548 */
static REAL CAT(layer_density, SFX)(const REAL* rhos, int layer, int maxl) {
    if (layer == 0) return 0.0;
    const int i = (layer <= maxl) ? layer - 1 : 2 * maxl - layer - 1;
    return rhos[i];
}

/*
 * Full CpuPropagator<REAL> evaluation.
 *   radii/rhos: n rows in any monotone order (propagator.hpp:117-161)
 *   result: AoS [n_cos][n_en][9], index in*3+out (physics.hpp:692-696)
 * Returns 0 on success, a negative code on the reference's error conditions.
 */
int CAT(oracle_calculate, SFX)(int n_cos, const REAL* cosines, int n_en, const REAL* energies,
                               int n_rows, const REAL* radii_in, const REAL* rhos_in,
                               REAL th12, REAL th13, REAL th23, REAL dcp,
                               REAL dm12sq, REAL dm23sq, REAL height_km, int anti,
                               int threads, REAL* result) {
    if (n_rows <= 0) return -1;  /* "vectors must not be empty" */
    REAL* radii = (REAL*)malloc(sizeof(REAL) * n_rows);
    REAL* rhos = (REAL*)malloc(sizeof(REAL) * n_rows);
    REAL* coslimit = (REAL*)malloc(sizeof(REAL) * n_rows);
    int* maxl = (int*)malloc(sizeof(int) * (n_cos > 0 ? n_cos : 1));
    int flip = 0;
    if (n_rows >= 2) {
        const int sign = (radii_in[1] - radii_in[0] > 0 ? 1 : -1);
        for (int i = 1; i < n_rows; i++)
            if ((radii_in[i] - radii_in[i - 1]) * sign < 0) {
                free(radii); free(rhos); free(coslimit); free(maxl);
                return -2;  /* "radii order messed up" */
            }
        if (sign == 1) flip = 1;
    }
    for (int i = 0; i < n_rows; i++) {
        const int src = flip ? n_rows - 1 - i : i;
        radii[i] = radii_in[src];
        rhos[i] = rhos_in[src];
    }
    for (int i = 0; i < n_rows; i++) {
        REAL x = -1 * sqrt(1 - (radii[i] * radii[i] / (K_REARTH * K_REARTH)));
        if (i == 0) x = 0;
        coslimit[i] = x;
    }
    for (int ic = 0; ic < n_cos; ic++) {
        const REAL c = cosines[ic];
        int cnt = 0;
        for (int i = 0; i < n_rows; i++) cnt += (c < coslimit[i]);
        maxl[ic] = cnt;
    }
    OSC st;
    CAT(set_mns, SFX)(&st, th12, th13, th23, dcp);
    CAT(set_masses, SFX)(&st, dm12sq, dm23sq);
    CAT(build_axfac, SFX)(&st);
    CAT(vacuum_order, SFX)(&st);
    const REAL hcm = height_km * 100000.0;
    const REAL REcm = K_REARTH * K_KM2CM;
    if (threads > 0) omp_set_num_threads(threads);

#pragma omp parallel for schedule(dynamic)
    for (int ic = 0; ic < n_cos; ic++) {
        const REAL c = cosines[ic];
        const REAL path = sqrt((REcm + hcm) * (REcm + hcm) - (REcm * REcm) * (1 - c * c)) - REcm * c;
        const REAL earth = -2.0 * c * REcm;
        const int M = maxl[ic];
        CPLX TM[3][3], CtM[3][3], F[3][3], T[3][3];
        for (int ie = 0; ie < n_en; ie++) {
            const REAL E = energies[ie];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) { CtM[i][j].re = (i == j ? 1.0 : 0.0); CtM[i][j].im = 0.0; }
            for (int l = 0; l <= M; l++) {
                const REAL dist = CAT(layer_distance, SFX)(radii, l, M, path, earth, c);
                const REAL dens = CAT(layer_density, SFX)(rhos, l, M);
                CAT(layer_amplitude, SFX)(&st, anti, E, dens * K_DENSCONV, dist / K_KM2CM, TM);
                if (l == 0) {
                    CAT(cmat_copy, SFX)(TM, F);
                } else if (l < M) {
                    CAT(cmat_zero, SFX)(T); CAT(cmat_mul_acc, SFX)(TM, F, T); CAT(cmat_copy, SFX)(T, F);
                    CAT(cmat_zero, SFX)(T); CAT(cmat_mul_acc, SFX)(CtM, TM, T); CAT(cmat_copy, SFX)(T, CtM);
                } else {
                    CAT(cmat_zero, SFX)(T); CAT(cmat_mul_acc, SFX)(TM, F, T); CAT(cmat_copy, SFX)(T, F);
                }
            }
            CAT(cmat_zero, SFX)(T); CAT(cmat_mul_acc, SFX)(CtM, F, T); CAT(cmat_copy, SFX)(T, F);
            REAL* out = result + ((size_t)ic * (size_t)n_en + (size_t)ie) * 9;
            for (int in = 0; in < 3; in++)
                for (int o = 0; o < 3; o++) {
                    const REAL re = F[o][in].re, im = F[o][in].im;
                    out[in * 3 + o] = re * re + im * im;
                }
        }
    }
    free(radii); free(rhos); free(coslimit); free(maxl);
    return 0;
}

/* Host-side pieces exposed for unit tests: maxlayers (propagator.hpp:301-307). */
int CAT(oracle_maxlayers, SFX)(int n_cos, const REAL* cosines, int n_rows, const REAL* radii_in,
                               int* maxl_out) {
    if (n_rows <= 0) return -1;
    const int asc = (n_rows >= 2 && radii_in[1] - radii_in[0] > 0);
    for (int ic = 0; ic < n_cos; ic++) {
        int cnt = 0;
        for (int i = 0; i < n_rows; i++) {
            const REAL r = radii_in[asc ? n_rows - 1 - i : i];
            REAL x = -1 * sqrt(1 - (r * r / (K_REARTH * K_REARTH)));
            if (i == 0) x = 0;
            cnt += (cosines[ic] < x);
        }
        maxl_out[ic] = cnt;
    }
    return 0;
}

#undef CPLX
#undef OSC
#undef U_
#undef DM_
#undef AX_
#undef K_GF
#undef K_KM2CM
#undef K_REARTH
#undef K_DENSCONV

/*
 * Oracle: CPU restatement of CUDAProb3++'s CpuPropagator path (double and float).
 *
 * TEST INFRASTRUCTURE ONLY.  It is the oracle of the CUDA library: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
 * load it.  The product path (cudaprob3_gb300) never links or calls it.
 *
 * Parity of this restatement with the reference itself is pinned by the golden
 * vectors in tests/golden/, which were produced by the reference's own
 * CpuPropagator<double> compiled from its headers (oracle/ref_shim.cpp).
 *
 * Built with -ffp-contract=off so that x86-64 and aarch64 evaluate the same
 * IEEE operations in the same order as the reference's host build.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdlib.h>
#include <omp.h>

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

#define REAL double
#define SFX _f64
#include "barger_oracle_body.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX _f32
#include "barger_oracle_body.h"
#undef REAL
#undef SFX

int oracle_abi_version(void) { return 1; }
int oracle_max_threads(void) { return omp_get_max_threads(); }

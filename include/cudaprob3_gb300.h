/*
 * cudaprob3_gb300 -- C ABI of the GB300 (sm_103a) Barger propagator.
 *
 * This is the drop-in boundary for CUDAProb3++'s single-GPU path: every entry
 * point below replaces one member of cudaprob3::CudaPropagatorSingle<FLOAT_T>
 * (cudapropagator.cuh:39-251) or of its base cudaprob3::Propagator<FLOAT_T>
 * (propagator.hpp:43-337).  The citation beside each declaration names the
 * reference member it replaces.  The C++ classes in include/cudaprob3/ wrap
 * this ABI with the reference's own class names and signatures.
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, doubles.  Host arrays are read
 *     during the call and not retained.
 *   - Every function returns CP3_OK (0) or a negative status.  The message of
 *     the last failure on the calling thread is returned by cp3_last_error().
 *     Where the reference throws std::runtime_error the same message text is
 *     used; where it calls exit(1) on a CUDA error (hpc_helpers.cuh:70-82)
 *     this ABI returns CP3_ERR_CUDA instead.
 *   - Each handle owns its device buffers, its stream and its parameters; no
 *     process-global physics state exists (the reference keeps its mixing
 *     data in globals, physics.hpp:114-124), so distinct handles may be used
 *     from distinct host threads.  One handle must not be used by two host
 *     threads at once.
 *   - Results live on the device in the reference's GPU layout: 9 planes
 *     [in*3+out][n_cosines][n_energies] (physics.hpp:689-691).  The element
 *     type is double for CP3_PRECISION_FP64 and float for CP3_PRECISION_MIXED.
 */
#ifndef CUDAPROB3_GB300_H
#define CUDAPROB3_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CP3_ABI_VERSION 1

/* status codes */
#define CP3_OK 0
#define CP3_ERR_ARGUMENT (-1)  /* bad size, index, pointer or value          */
#define CP3_ERR_STATE (-2)     /* call order violated / input not yet set     */
#define CP3_ERR_CUDA (-3)      /* CUDA runtime failure                         */
#define CP3_ERR_NO_DEVICE (-4) /* no GPU, or the device id does not exist     */
#define CP3_ERR_FILE (-5)      /* density file could not be opened            */
#define CP3_ERR_LIMIT (-6)     /* a size exceeds a documented limit           */
#define CP3_ERR_CHECK (-7)     /* bounds-checked build: a kernel index failed  */

/* arithmetic of a propagator */
#define CP3_PRECISION_FP64 0  /* plain method: every step in FP64              */
#define CP3_PRECISION_MIXED 1 /* double-float eigen-solve, 32-bit bulk, float results */

/* NeutrinoType, types.hpp:29 */
#define CP3_NEUTRINO 0
#define CP3_ANTINEUTRINO 1

/* ProbType index = in*3+out, types.hpp:23-27 */

typedef struct cp3_propagator cp3_propagator;

/* Version of this ABI (CP3_ABI_VERSION). */
int cp3_abi_version(void);

/* 1 in the bounds-checked debug build (libcudaprob3_gb300_check.so, compiled
 * with -DCP3_CHECK), 0 otherwise.  No reference counterpart: the reference
 * indexes its device arrays unchecked (physics.hpp:689-696).  In the checked
 * build every shared- and global-memory index of the kernels is compared with
 * its buffer's extent; a failure is recorded (never a trap), the access is
 * kept inside the buffer, and the wait that ends the calculation
 * (cp3_wait_for_completion, cp3_batch_wait, cp3_loglik_evaluate, and the
 * no-allocation call, which waits in the checked build) returns CP3_ERR_CHECK with
 * the kernel, index and extent in cp3_last_error(). */
int cp3_bounds_checked(void);

/* Message of the last failure on this thread ("" when none). */
const char* cp3_last_error(void);

/* Number of visible CUDA devices (0 when none); never fails. */
int cp3_device_count(void);

/* CudaPropagatorSingle(int id, int n_cosines, int n_energies),
 * cudapropagator.cuh:50-80; `precision` selects the arithmetic. */
int cp3_create(cp3_propagator** out, int device_id, int n_cosines, int n_energies,
               int precision);

/* ~CudaPropagatorSingle(), cudapropagator.cuh:91-94.  NULL is accepted. */
int cp3_destroy(cp3_propagator* p);

/* Propagator::setEnergyList, propagator.hpp:252-257 (GeV); n must equal n_energies. */
int cp3_set_energy_list(cp3_propagator* p, const double* energies, int n);

/* Propagator::setCosineList, propagator.hpp:261-274; n must equal n_cosines. */
int cp3_set_cosine_list(cp3_propagator* p, const double* cosines, int n);

/* Propagator::setMNSMatrix, propagator.hpp:191-221 (radians). */
int cp3_set_mns_matrix(cp3_propagator* p, double theta12, double theta13, double theta23,
                       double dcp);

/* Propagator::setNeutrinoMasses, propagator.hpp:226-248 (eV^2). */
int cp3_set_neutrino_masses(cp3_propagator* p, double dm12sq, double dm23sq);

/* Propagator::setDensity, propagator.hpp:117-161 (km, g/cm^3), extended by an
 * electron fraction per row.  `ye` may be NULL: every row then uses 0.5, the
 * reference's fixed factor (constants.hpp:40).  Rows: 1..CP3_MAX_ROWS. */
int cp3_set_density(cp3_propagator* p, const double* radii, const double* rhos,
                    const double* ye, int n);
#define CP3_MAX_ROWS 64

/* Propagator::setDensityFromFile, propagator.hpp:169-184 (two columns). */
int cp3_set_density_from_file(cp3_propagator* p, const char* path);

/* Propagator::setProductionHeight, propagator.hpp:279-286 (km). */
int cp3_set_production_height(cp3_propagator* p, double height_km);

/* Production-height distribution (no reference counterpart: the reference
 * takes one height, propagator.hpp:279-286).  Probabilities are averaged over
 * the n heights (km, >= 0) with the given weights (>= 0, normalised here):
 *   P(c, E) = sum_h w_h P(c, E; h).
 * Only the atmosphere segment depends on the height, so the layer chain runs
 * once per pair and each height adds one phase pair and a 2x3 by 3x2 product.
 * n = 1 is cp3_set_production_height; cp3_set_production_height ends the
 * distribution.  Fused rates are not available with a distribution. */
#define CP3_MAX_HEIGHTS 64
int cp3_set_production_heights(cp3_propagator* p, const double* heights_km, const double* weights, int n);

/* CudaPropagatorSingle::calculateProbabilities, cudapropagator.cuh:162-165
 * (launch and wait).  type: CP3_NEUTRINO or CP3_ANTINEUTRINO. */
int cp3_calculate_probabilities(cp3_propagator* p, int type);

/* CudaPropagatorSingle::calculateProbabilitiesAsync, cudapropagator.cuh:191-220. */
int cp3_calculate_probabilities_async(cp3_propagator* p, int type);

/* CudaPropagatorSingle::waitForCompletion, cudapropagator.cuh:223-226. */
int cp3_wait_for_completion(cp3_propagator* p);

/* CudaPropagatorSingle::getProbability, cudapropagator.cuh:168-181.  The first
 * call after a calculation copies all 9 planes to pinned host memory. */
int cp3_get_probability(cp3_propagator* p, int index_cosine, int index_energy,
                        int prob_type, double* out);

/* Device pointer of the result planes (no reference counterpart: the
 * reference keeps d_result_list private, cudapropagator.cuh:245). */
int cp3_result_device_ptr(cp3_propagator* p, void** dptr);

/* Size in bytes of the result planes: 9 * n_cosines * n_energies * element. */
int cp3_result_bytes(cp3_propagator* p, size_t* bytes);

/* Copy all result planes to host memory `dst` of `bytes` bytes
 * (cudapropagator.cuh:229-235 without the lazy flag). */
int cp3_copy_results_to_host(cp3_propagator* p, void* dst, size_t bytes);

/* Write results into a caller-owned device buffer (>= cp3_result_bytes) from
 * the next calculation on; NULL returns to the handle's own buffer. */
int cp3_set_result_buffer(cp3_propagator* p, void* dptr, size_t bytes);

/* Zero-copy host results (no reference counterpart: the reference copies
 * d_result_list into its pinned resultList on the first getProbability after
 * a calculation, cudapropagator.cuh:168-181 and 228-234).  `host` must be page-locked (cudaHostAlloc or
 * cudaHostRegister) and hold >= cp3_result_bytes; from the next calculation on
 * the kernel stores the planes straight into it over the host link, so the
 * transfer overlaps the computation.  cp3_get_probability then reads it
 * without a copy.  Pageable memory is rejected with CP3_ERR_ARGUMENT; NULL
 * returns to the handle's own device buffer. */
int cp3_set_host_result_buffer(cp3_propagator* p, void* host, size_t bytes);

/* With a host result buffer: enable = 1 makes the kernel store only the four
 * planes of the 2x2 flavour block (e->e, e->mu, mu->e, mu->mu: 4/9 of the
 * bytes over the host link) and cp3_wait_for_completion derive the other five
 * on the host cores from unitarity (rows and columns sum to one; in double,
 * one rounding, clamped at zero).  The four stored planes are the kernel's;
 * the derived ones differ from the device completion by a few units of the
 * last place.  No effect without a host result buffer, with fused rates or
 * with a production-height distribution.  Default 0.  (No reference
 * counterpart.) */
int cp3_set_host_completion(cp3_propagator* p, int enable);

/* ---- Fused event rates (no reference counterpart) -------------------------
 * The reference's caller reads all nine planes back (getProbability,
 * cudapropagator.cuh:168-181) to weight events.  These entry points do that
 * weighting inside the propagation kernel, so the planes never leave the SM:
 *   rate_b(c, E) = sum_a flux[a][c][E] * P(a -> b)(c, E),   a, b in (e, mu, tau)
 *   hist[b][cos_bin[c]][en_bin[E]] += rate_b(c, E)
 * FP64 histograms; within a histogram bin the order of the additions is not
 * fixed (atomics), so results can differ in the last bits between runs. */

/* Flux (any per-(cosine, energy) weight: flux x cross-section x exposure ...)
 * [3][n_cosines][n_energies] floats, plane a = initial flavour a.  Only planes
 * whose bit is set in flavour_mask (1 = e, 2 = mu, 4 = tau) are read; the
 * others count as zero.  on_device = 0: host memory, copied now; 1: a device
 * pointer the handle keeps using (caller-owned, must outlive the handle's
 * calculations). */
int cp3_set_rate_flux(cp3_propagator* p, const float* flux, int flavour_mask, int on_device);

/* Histogram binning: cos_bin[n_cosines] in [-1, n_cos_bins), en_bin[n_energies]
 * in [-1, n_en_bins); -1 leaves that cosine / energy out.  Monotone bins (each
 * bin a contiguous range) are the fast case; any assignment is correct. */
int cp3_set_rate_bins(cp3_propagator* p, const int* cos_bin, const int* en_bin, int n_cos_bins, int n_en_bins);

/* One propagation into the histograms [3][n_cos_bins][n_en_bins] (zeroed
 * first); the nine planes are not written.  Same preconditions as
 * cp3_calculate_probabilities, plus flux and bins. */
int cp3_calculate_rates(cp3_propagator* p, int type);
int cp3_calculate_rates_async(cp3_propagator* p, int type);

/* Device pointer of the histograms, and a synchronous copy of them into host
 * memory (count >= 3 * n_cos_bins * n_en_bins doubles). */
int cp3_rates_device_ptr(cp3_propagator* p, double** dptr);
int cp3_get_rates(cp3_propagator* p, double* host, size_t count);

/* Run on a caller-owned cudaStream_t (NULL returns to the handle's own stream). */
int cp3_set_stream(cp3_propagator* p, void* cuda_stream);

/* Kernel launches issued by the last calculation (all are this library's). */
int cp3_last_launch_count(cp3_propagator* p, int* launches);

/* Launch shape of the propagate kernel: energies per tile te (32, 64, 128),
 * cosine groups per block, cosines per block (no reference counterpart: the
 * reference launches 64-thread blocks, cudapropagator.cuh:204-209). */
int cp3_set_launch_shape(cp3_propagator* p, int te, int groups, int cchunk);
int cp3_get_launch_shape(cp3_propagator* p, int* te, int* groups, int* cchunk);
/* Times every supported launch shape on `reps` calculations of this handle's
 * grid and keeps the fastest (the results of the calculations are valid). */
int cp3_autotune(cp3_propagator* p, int type, int reps, int* te, int* groups, int* cchunk,
                 float* best_ms);

/* Layers crossed per cosine (Propagator::maxlayers, propagator.hpp:301-307). */
int cp3_get_maxlayers(cp3_propagator* p, int* out, int n);

/* Record CUDA events around each kernel of the following calculations
 * (0 disables); cp3_last_kernel_ms returns the durations of the last one. */
int cp3_set_kernel_timing(cp3_propagator* p, int enable);
int cp3_last_kernel_ms(cp3_propagator* p, float* prep_ms, float* propagate_ms);

/* ------------------------------------------------------------------ batches
 * Many independent propagations ("parameter sets") evaluated together: set s
 * has its own oscillation parameters, density scale and grid of
 * n_cosines[s] x n_energies[s] pairs, and its results are the reference's
 * [9][n_cosines[s]][n_energies[s]] planes at element offset offsets[s].  One
 * calculation is one CUDA-graph launch: a counter reset, then the sets in up
 * to 8 chunks of growing work, each an FP64 precompute kernel on a
 * low-priority branch and a persistent kernel on the high-priority one that
 * takes (set, energy tile, cosine chunk) work items, largest first; the
 * precompute of chunk k + 1 runs beside the propagation of chunk k.  No reference counterpart
 * (the reference evaluates one parameter point per calculateProbabilities).
 * Errors are reported through cp3_last_error() like the single-grid ABI. */
typedef struct cp3_batch cp3_batch;

int cp3_batch_create(cp3_batch** out, int device_id, int precision, int n_sets,
                     const int* n_cosines, const int* n_energies);
int cp3_batch_destroy(cp3_batch* b);
/* all sets' cosines, then all sets' energies, concatenated in set order */
int cp3_batch_set_grids(cp3_batch* b, const double* cosines, const double* energies);
/* params[6*s + k]: theta12, theta13, theta23, dcp (rad), dm12sq, dm23sq (eV^2) */
int cp3_batch_set_parameters(cp3_batch* b, const double* params);
/* one body for all sets; densities of set s multiplied by scale[s] (NULL: 1) */
int cp3_batch_set_density(cp3_batch* b, const double* radii, const double* rhos,
                          const double* ye, int n, const double* scale);
int cp3_batch_set_production_height(cp3_batch* b, double height_km);
int cp3_batch_set_stream(cp3_batch* b, void* cuda_stream);
/* energies per tile (32, 64, 128), cosine groups per block, cosines per item */
int cp3_batch_set_launch_shape(cp3_batch* b, int te, int groups, int cchunk);
int cp3_batch_get_launch_shape(cp3_batch* b, int* te, int* groups, int* cchunk, int* blocks);
/* times every supported launch shape on `reps` launches and keeps the fastest */
int cp3_batch_autotune(cp3_batch* b, int type, int reps, int* te, int* groups, int* cchunk,
                       float* best_ms);
int cp3_batch_calculate(cp3_batch* b, int type);
int cp3_batch_calculate_async(cp3_batch* b, int type);
int cp3_batch_wait(cp3_batch* b);
/* the same work as two single-grid launches per set (for comparison) */
int cp3_batch_calculate_sequential(cp3_batch* b, int type);
/* device time of the last calculation (events around the graph or launches) */
int cp3_batch_last_ms(cp3_batch* b, float* ms);
/* kernels one cp3_batch_calculate launches (the graph's prep and propagate
 * launches of every chunk, for the current sets and launch shape) */
int cp3_batch_launch_count(cp3_batch* b, int type, int* launches);
/* n_sets + 1 element offsets of each set's planes in the result buffer */
int cp3_batch_result_offsets(cp3_batch* b, long long* offsets);
int cp3_batch_result_device_ptr(cp3_batch* b, void** dptr);
int cp3_batch_copy_results_to_host(cp3_batch* b, void* dst, size_t bytes);
int cp3_batch_get_maxlayers(cp3_batch* b, int* out, long long n);

/* ------------------------------------------------------ log-likelihood
 * Binned Poisson log-likelihood of the propagated probabilities and its
 * gradient by a hand-written adjoint.  Bin (c, e) expects
 *   lambda = norm * (flux_e[e] P(e -> mu) + flux_mu[e] P(mu -> mu))
 * events and LL = sum n ln(lambda) - lambda.  The gradient is with respect to
 * theta12, theta13, theta23, dcp, dm12sq, dm23sq and the density of every row
 * of the body (in the order given to cp3_loglik_set_body).  The per-layer
 * matrices are recomputed in the backward pass, not stored.  No reference
 * counterpart (the reference computes probabilities only). */
typedef struct cp3_loglik cp3_loglik;

int cp3_loglik_create(cp3_loglik** out, int device_id, int precision, int n_cosines, int n_energies);
int cp3_loglik_destroy(cp3_loglik* L);
int cp3_loglik_set_bins(cp3_loglik* L, const double* cosines, const double* energies);
/* radii (any monotone order, as setDensity) and electron fractions (NULL: 0.5) */
int cp3_loglik_set_body(cp3_loglik* L, const double* radii, const double* ye, int n);
int cp3_loglik_set_production_height(cp3_loglik* L, double height_km);
int cp3_loglik_set_flux(cp3_loglik* L, const double* flux_e, const double* flux_mu, double norm);
/* observed counts, [n_cosines][n_energies] */
int cp3_loglik_set_observed(cp3_loglik* L, const double* counts);
/* params: theta12, theta13, theta23, dcp, dm12sq, dm23sq; rhos: one per row.
 * grad (may be NULL) receives 6 + n_rows values. */
int cp3_loglik_evaluate(cp3_loglik* L, int type, const double* params, const double* rhos,
                        double* loglik, double* grad);
/* Record CUDA events around each of the evaluation's three kernels (prep,
 * pair, layer) from the next evaluation on (0 disables; toggling recaptures
 * the evaluation graph); cp3_loglik_last_kernel_ms returns the durations of
 * the last evaluation. */
int cp3_loglik_set_kernel_timing(cp3_loglik* L, int enable);
int cp3_loglik_last_kernel_ms(cp3_loglik* L, float* prep_ms, float* pair_ms, float* layer_ms);
/* Bytes one evaluation moves between host and device: the parameter block
 * the graph uploads, and the per-energy log-likelihood and gradient rows the
 * layer kernel writes into mapped host memory (the body must be set). */
int cp3_loglik_io_bytes(cp3_loglik* L, long long* host_to_device, long long* device_to_host);

/* ------------------------------------------------------------- no allocation
 * One calculation that allocates nothing.  No counterpart in the reference.
 * It is for callers that cannot call cudaMalloc:
 *   - code inside a framework whose caching allocator owns (nearly) all device
 *     memory, so that an allocation behind its back can fail, and whose
 *     cudaFree would synchronise the whole device;
 *   - fitters evaluating thousands of parameter points per second, which
 *     cannot take that synchronisation inside their loop;
 *   - plugins that a host application hands only device pointers and a
 *     stream, and that may not own device memory.
 *
 * Runs on the current device and `stream` (NULL: the default stream).  Inputs
 * d_cosines[n_cosines] and d_energies[n_energies] and the output
 * d_out[9][n_cosines][n_energies] (float for CP3_PRECISION_MIXED, double for
 * CP3_PRECISION_FP64, plane in*3+out as cp3_result_device_ptr) are device
 * memory owned by the caller; radii/rhos/ye (ye may be NULL: 0.5) are host
 * arrays read during the call, with the checks and messages of
 * cp3_set_density.  The results are bit for bit those of cp3_create,
 * cp3_set_* and cp3_calculate_probabilities with the default launch shape on
 * the same inputs (production height set after the cosine list).
 * Scratch lives in one static device array sized for the limits below (about
 * 14 MB, held by every GPU that loads the library until the process exits);
 * larger problems are rejected with CP3_ERR_LIMIT, and nothing is allocated
 * (no cudaMalloc, cudaFree or allocating library call).  The first call on a
 * device sets that device up: it looks up the array's device address
 * (cudaGetSymbolAddress) and copies the phase tables into it synchronously
 * (the only host-synchronous step of the call).  Every call shares the
 * array, which keeps the last call's contents; each call rewrites what it
 * reads before reading it, but calls whose work overlaps on the GPU (other
 * streams or host threads) race on it and must be serialised by the caller.
 * After the set-up the call is asynchronous with respect to the host. */
#define CP3_NOALLOC_MAX_COSINES 8192
#define CP3_NOALLOC_MAX_ENERGIES 8192
#define CP3_NOALLOC_MAX_ROWS 15
int cp3_propagate_noalloc(int precision, int type, const double* d_cosines, int n_cosines,
                          const double* d_energies, int n_energies, const double* radii,
                          const double* rhos, const double* ye, int n_rows, double theta12,
                          double theta13, double theta23, double dcp, double dm12sq,
                          double dm23sq, double height_km, void* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CUDAPROB3_GB300_H */

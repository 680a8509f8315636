// Test infrastructure only: the reference's own CUDA kernel,
// calculateKernel<FLOAT_T> (physics.hpp:705-721, launched by
// CudaPropagatorSingle with 64-thread blocks and SDIV(n_energies, 64) *
// n_cosines blocks, cudapropagator.cuh:191-220), compiled from the reference's
// headers where they lie into a cubin for sm_103a (oracle/Makefile, target
// refgpu; output oracle/_ref/, never committed): the reference's GPU path
// recompiled for this GPU, the comparison for the propagation kernels on the
// same device.  Nothing in the product loads it; bench.py times it through
// oracle/ref_gpu_driver.cpp.
// the include order of cudapropagator.cuh:23-26
#include "constants.hpp"
#include "propagator.hpp"
#include "physics.hpp"

namespace cudaprob3 {
namespace physics {

template __global__ void calculateKernel<double>(NeutrinoType, const double* const, int, const double* const, int,
                                                 const double* const, const double* const, const int* const, double,
                                                 double* const);
template __global__ void calculateKernel<float>(NeutrinoType, const float* const, int, const float* const, int,
                                                const float* const, const float* const, const int* const, float,
                                                float* const);

}  // namespace physics
}  // namespace cudaprob3

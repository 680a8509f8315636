// Umbrella header of the C++ drop-in API.
#ifndef CUDAPROB3_GB300_ALL_HPP
#define CUDAPROB3_GB300_ALL_HPP
#include "cudapropagator.hpp"
#include "propagator.hpp"
#include "types.hpp"
#endif

"""GB300-native (sm_103a) Barger propagator with CUDAProb3++'s interface.

The compute path is libcudaprob3_gb300.so (hand-written CUDA kernels behind a
C ABI, include/cudaprob3_gb300.h).  ``CudaPropagatorSingle`` mirrors the
reference's class of the same name; ``grids`` holds the example grids and
bodies.
"""
from ._lib import CP3Error, load as load_library  # noqa: F401
from .propagator import (Antineutrino, CudaPropagatorSingle, Neutrino, NeutrinoType,  # noqa: F401
                         ProbType, device_count)

__all__ = ["CudaPropagatorSingle", "NeutrinoType", "ProbType", "Neutrino", "Antineutrino",
           "CP3Error", "device_count", "load_library"]

"""Oracle package: the CPU oracle of the CUDA library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference arms (the CPU port, and the reference's own kernel on the GPU)
import this package.  The product (``cudaprob3_gb300``) never
imports it; there is no CPU fallback in the product path.

* ``calculate``      -- the C restatement of the reference's CpuPropagator
                        (barger_oracle_body.h), double or float.
* ``ref_calculate``  -- the reference's own CpuPropagator compiled from its
                        headers (oracle/_ref/libcp3ref.so), present only where
                        the reference sources were available at build time;
                        ``ref_calculate_file`` reads the body with its
                        setDensityFromFile.
* ``ref_gpu_run``    -- the reference's own CUDA kernel (calculateKernel,
                        compiled for sm_103a into oracle/_ref) launched on the
                        benchmark grid with the inputs its host code prepared
                        (bench.py's GPU comparison).
"""
from .oracle import (build, calculate, ref_calculate, ref_calculate_file, ref_available, ref_gpu_run,
                     ref_gpu_status, maxlayers, max_threads)

__all__ = ["build", "calculate", "ref_calculate", "ref_calculate_file", "ref_available", "ref_gpu_run",
           "ref_gpu_status", "maxlayers", "max_threads"]

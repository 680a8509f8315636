"""Oracle package: the checker for the CUDA library (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference arms import this package.  The product (``cudaprob3_gb300``) never
imports it; there is no CPU fallback in the product path.

* ``calculate``      -- the C restatement of the reference's CpuPropagator
                        (barger_oracle_body.h), double or float.
* ``ref_calculate``  -- the reference's own CpuPropagator compiled from its
                        headers (oracle/_ref/libcp3ref.so), present only where
                        the reference sources were available at build time.
"""
from .oracle import (build, calculate, ref_calculate, ref_available, maxlayers,
                     max_threads)

__all__ = ["build", "calculate", "ref_calculate", "ref_available", "maxlayers",
           "max_threads"]

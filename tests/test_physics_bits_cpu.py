"""Host build of the kernels' bit-level helpers and eigen-solve
(cudaprob3_gb300/csrc/cp3_physics.cuh compiled with g++): the integer-pipe
conversions equal the hardware conversions they replace (Q1.30 rounding half
to even, double to float and back, with the documented flush below FLT_MIN),
the cm-to-km FMA correction equals the division, div_nr is within one ulp,
the bit-pattern compares order like the FP64 compares, and the eigen-solve
returns right-handed orthonormal eigen-pairs of 2E*H_r (200,000 random
parameter sets with degeneracies, both orderings and vacuum layers:
|HV - Vm| / |H| <= 1e-11, |V^T V - I| <= 1e-14, det V = 1)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "physics_bits_check.cpp")


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_physics_helpers_host_build(tmp_path):
    exe = str(tmp_path / "physics_bits_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "cudaprob3_gb300", "csrc"),
                    SRC, "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe, "1000000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert r.stdout.strip().endswith("bad 0")

"""The C++ drop-in API (include/cudaprob3/) compiled like the reference's
example driver and run on the GPU; results compared with the oracle."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import _lib
from cudaprob3_gb300 import grids as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp")


def compile_example(outdir):
    exe = os.path.join(outdir, "dropin_example")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++14", "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L" + libdir, "-lcudaprob3_gb300", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_cpp_api_compiles():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.fail("libcudaprob3_gb300.so is not built")
    with tempfile.TemporaryDirectory() as d:
        assert os.path.exists(compile_example(d))


@pytest.mark.gpu
def test_cpp_dropin_runs_like_reference_example(gpu):
    nc, ne = 37, 45
    with tempfile.TemporaryDirectory() as d:
        exe = compile_example(d)
        dens = os.path.join(d, "prem12.dat")
        with open(dens, "w") as f:
            for r, rho in zip(G.PREM_12.radii, G.PREM_12.rhos):
                f.write("%.17g %.17g\n" % (r, rho))
        out = os.path.join(d, "out.bin")
        r = subprocess.run([exe, out, dens], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        raw = np.fromfile(out, dtype=np.float64)
    per = nc + ne + nc * ne * 9
    assert raw.size == 4 * per
    B = G.PREM_12
    for k, (tol, f32) in enumerate(((1e-11, False), (1e-6, True), (1e-11, False), (1e-6, True))):
        blk = raw[k * per:(k + 1) * per]
        c, e = blk[:nc], blk[nc:nc + ne]
        got = blk[nc + ne:].reshape(nc, ne, 9)
        # the float API reads the density file and the parameters as floats
        cast = (lambda x: np.asarray(x, dtype=np.float32).astype(np.float64)) if f32 else np.asarray
        params = tuple(float(cast(x)) for x in G.NOMINAL)
        want = oracle.calculate(c, e, cast(B.radii), cast(B.rhos), params, float(cast(22.0)), False,
                                planar=False)
        assert np.abs(got - want).max() <= tol, "propagator %d: %.3g" % (k, np.abs(got - want).max())

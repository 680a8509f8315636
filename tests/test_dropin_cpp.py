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
EXT = os.path.join(ROOT, "tests", "cpp", "extensions_example.cpp")


def compile_example(outdir, src=SRC):
    exe = os.path.join(outdir, os.path.splitext(os.path.basename(src))[0])
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++14", "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
           "-L" + libdir, "-lcudaprob3_gb300", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_cpp_api_compiles():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.fail("libcudaprob3_gb300.so is not built")
    with tempfile.TemporaryDirectory() as d:
        assert os.path.exists(compile_example(d))
        assert os.path.exists(compile_example(d, EXT))


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
    assert raw.size == 6 * per
    B = G.PREM_12
    # Single<double>, Single<float>, CudaPropagator<double>({0,0}), <float>({0}),
    # <double>({0}), <double>({0,0,0})
    kinds = ((1e-11, False), (1e-6, True), (1e-11, False), (1e-6, True), (1e-11, False), (1e-11, False))
    for k, (tol, f32) in enumerate(kinds):
        blk = raw[k * per:(k + 1) * per]
        c, e = blk[:nc], blk[nc:nc + ne]
        got = blk[nc + ne:].reshape(nc, ne, 9)
        # the float API reads the density file and the parameters as floats
        cast = (lambda x: np.asarray(x, dtype=np.float32).astype(np.float64)) if f32 else np.asarray
        params = tuple(float(cast(x)) for x in G.NOMINAL)
        want = oracle.calculate(c, e, cast(B.radii), cast(B.rhos), params, float(cast(22.0)), False,
                                planar=False)
        assert np.abs(got - want).max() <= tol, "propagator %d: %.3g" % (k, np.abs(got - want).max())


@pytest.mark.gpu
def test_cpp_extensions_heights_and_rates(gpu):
    """setProductionHeights and the fused rates through the C++ classes,
    against the oracle (FP64 handle: 1e-11 on probabilities, 1e-12 relative on
    the histograms)."""
    nc, ne = 21, 17
    with tempfile.TemporaryDirectory() as d:
        exe = compile_example(d, EXT)
        out = os.path.join(d, "out.bin")
        r = subprocess.run([exe, out], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        raw = np.fromfile(out, dtype=np.float64)
    assert raw.size == nc * ne * 9 + 60
    c = -1.0 + 1.5 * np.arange(nc) / (nc - 1)
    e = 0.5 * 100.0 ** (np.arange(ne) / (ne - 1))
    radii = [0.0, 1220.0, 3480.0, 5701.0, 6371.0]
    rhos = np.array([13.0, 13.0, 11.3, 5.0, 3.3])
    avg = sum(w * oracle.calculate(c, e, radii, rhos, G.NOMINAL, h, False, planar=False)
              for h, w in ((10.0, 0.25), (20.0, 0.5), (30.0, 0.25)))
    assert np.abs(raw[:nc * ne * 9].reshape(nc, ne, 9) - avg).max() <= 1e-11
    P = oracle.calculate(c, e, radii, rhos, G.NOMINAL, 22.0, False)  # [9][nc][ne]
    rate = np.stack([1.0 * P[0 + b] + 2.0 * P[3 + b] for b in range(3)])
    cb = np.arange(nc) * 4 // nc
    eb = np.arange(ne) * 5 // ne
    want = np.zeros((3, 4, 5))
    for b in range(3):
        np.add.at(want[b], (cb[:, None].repeat(ne, 1), eb[None, :].repeat(nc, 0)), rate[b])
    got = raw[nc * ne * 9:].reshape(3, 4, 5)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()

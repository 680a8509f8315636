"""The bounds-checked debug build (libcudaprob3_gb300_check.so, the same sources
compiled with -DCP3_CHECK) on the cases whose indexing is most irregular:
ragged grid sizes, the 60-row body that makes the handle halve its energy tile
and the batch use two-warp prep blocks, an empty grid, fused rates,
production-height averages, the batch, the log-likelihood and the
no-allocation call.  Every kernel index is compared with its buffer's extent
there; a failed check would make the calculation return CP3_ERR_CHECK.  The
build runs in a child process (the library is chosen when the package is first
loaded), and its results are also checked against the oracle.
"""
import os
import subprocess
import sys

import pytest

from cudaprob3_gb300 import _lib

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import ctypes, os, sys
import numpy as np
sys.path.insert(0, os.environ["CP3_TEST_ROOT"])
sys.path.insert(0, os.path.join(os.environ["CP3_TEST_ROOT"], "tests"))
import oracle
import cudaprob3_gb300 as cp
from cudaprob3_gb300 import _lib, grids as G
lib = _lib.load()
assert lib.cp3_bounds_checked() == 1, "not the checked build"
TOL = {"fp64": 1e-11, "mixed": 1e-6}

def run(precision, cos, en, B, params=G.NOMINAL, anti=False):
    with cp.CudaPropagatorSingle(0, len(cos), len(en), precision=precision) as p:
        p.setEnergyList(en); p.setCosineList(cos)
        p.setMNSMatrix(*params[:4]); p.setNeutrinoMasses(*params[4:])
        p.setDensity(B.radii, B.rhos, B.ye); p.setProductionHeight(22.0)
        p.calculateProbabilities(cp.Antineutrino if anti else cp.Neutrino)
        return p.results().astype(np.float64)

# ragged sizes and upgoing cosines
for precision in ("fp64", "mixed"):
    for nc, ne in [(1, 1), (1, 37), (3, 1), (5, 129), (130, 7), (37, 53)]:
        c = G.linspace(-1, 0.5, nc) if nc > 1 else np.array([-0.7])
        e = G.logspace(0.2, 200, ne) if ne > 1 else np.array([3.0])
        got = run(precision, c, e, G.PREM_12)
        want = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL)
        assert np.abs(got - want).max() <= TOL[precision], (precision, nc, ne)
print("ragged ok", flush=True)

# 60 rows: the energy tile is halved to fit shared memory
r59, d59 = G.read_density_file(os.path.join(os.environ["CP3_TEST_ROOT"], "tests", "golden", "models",
                                            "PREM_59layer.dat"))
B59 = G.Body(r59, d59, np.where(r59 <= 3480.0, 0.468, 0.497))
c, e = G.linspace(-1, 0, 70), G.logspace(0.1, 1000, 90)
for precision in ("fp64", "mixed"):
    got = run(precision, c, e, B59)
    want = oracle.calculate(c, e, B59.radii, B59.rho_eff(), G.NOMINAL)
    assert np.abs(got - want).max() <= TOL[precision], precision
print("60 rows ok", flush=True)

# empty grid
with cp.CudaPropagatorSingle(0, 0, 16) as p:
    p.setEnergyList(G.logspace(1, 10, 16)); p.setCosineList([])
    p.setMNSMatrix(*G.NOMINAL[:4]); p.setNeutrinoMasses(*G.NOMINAL[4:])
    p.setDensity(G.PREM_4.radii, G.PREM_4.rhos); p.setProductionHeight(22.0)
    p.calculateProbabilities(cp.Neutrino)

# fused rates and production-height averages
nc, ne = 41, 67
c, e = G.linspace(-1, 0.2, nc), G.logspace(0.5, 100, ne)
for precision in ("fp64", "mixed"):
    with cp.CudaPropagatorSingle(0, nc, ne, precision=precision) as p:
        p.setEnergyList(e); p.setCosineList(c)
        p.setMNSMatrix(*G.NOMINAL[:4]); p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye); p.setProductionHeight(22.0)
        flux = np.ones((3, nc, ne), np.float32)
        p.setRateFlux(flux, 7)
        p.setRateBins((np.arange(nc) * 5) // nc, (np.arange(ne) * 7) // ne, 5, 7)
        hist = p.calculateRates(cp.Neutrino)
        assert np.isfinite(hist).all()
        p.setProductionHeights([10.0, 20.0, 30.0], [0.25, 0.5, 0.25])
        p.calculateProbabilities(cp.Neutrino)
        avg = sum(w * oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, h, False)
                  for h, w in ((10.0, 0.25), (20.0, 0.5), (30.0, 0.25)))
        assert np.abs(p.results().astype(np.float64) - avg).max() <= TOL[precision], precision
print("rates and heights ok", flush=True)

# batch: 12-row and 60-row bodies, graph and sequential launches
from test_batch_gpu import make_sets
from cudaprob3_gb300.batch import BatchPropagator
for body in (G.PREM_12, B59):
    for precision in ("mixed", "fp64"):
        nc_s, ne_s, params, scale, cos_s, en_s = make_sets(6, seed=11)
        with BatchPropagator(0, nc_s, ne_s, precision=precision) as b:
            b.set_grids(cos_s, en_s); b.set_parameters(params)
            b.set_density(body.radii, body.rhos, body.ye, scale); b.set_production_height(22.0)
            for seq in (False, True):
                (b.calculate_sequential if seq else b.calculate)(0)
                flat = b.results()
                for s in range(len(nc_s)):
                    got = b.set_result(flat, s).astype(np.float64)
                    want = oracle.calculate(cos_s[s], en_s[s], body.radii, body.rho_eff() * scale[s],
                                            tuple(params[s]), 22.0, False)
                    assert np.abs(got - want).max() <= TOL[precision], (precision, s, seq)
print("batch ok", flush=True)

# log-likelihood and its gradient
from cudaprob3_gb300.loglik import binned_problem
prob = binned_problem(n_cos=64, n_en=40)
for precision in ("fp64", "mixed"):
    L = prob.make(device_id=0, precision=precision)
    ll, g = L.evaluate(prob.nominal, prob.body.rhos)
    assert np.isfinite(ll) and np.isfinite(g).all()
    L.close()
print("loglik ok", flush=True)

# the no-allocation call (waits in the checked build and reports its checks)
import torch
c, e = G.linspace(-1, 0.2, 300), G.logspace(0.1, 1000, 257)
dc = torch.tensor(c, dtype=torch.float64, device="cuda:0")
de = torch.tensor(e, dtype=torch.float64, device="cuda:0")
out = torch.empty((9, 300, 257), dtype=torch.float32, device="cuda:0")
r, d, y = [np.ascontiguousarray(a, dtype=np.float64) for a in (G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye)]
dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
rc = lib.cp3_propagate_noalloc(1, 0, ctypes.c_void_p(dc.data_ptr()), 300, ctypes.c_void_p(de.data_ptr()), 257,
                               dp(r), dp(d), dp(y), int(r.size), *[float(x) for x in G.NOMINAL], 22.0,
                               ctypes.c_void_p(out.data_ptr()), None)
assert rc == 0, lib.cp3_last_error().decode()
want = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL)
assert np.abs(out.double().cpu().numpy() - want).max() <= 1e-6
print("CHECKED_OK", flush=True)
'''


def test_checked_build_runs_the_irregular_cases_clean(gpu):
    if not os.path.exists(_lib.CHECK_LIB_PATH):
        pytest.fail("libcudaprob3_gb300_check.so is not built (cudaprob3_gb300.build builds it)")
    env = dict(os.environ, CUDAPROB3_GB300_LIBRARY=_lib.CHECK_LIB_PATH, CP3_TEST_ROOT=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "CHECKED_OK" in r.stdout, (r.stdout[-2000:], r.stderr[-3000:])

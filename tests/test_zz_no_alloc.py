"""The entry point that allocates nothing, cp3_propagate_noalloc, against the
regular handle path (cp3_create ... cp3_calculate_probabilities).

It serves callers that cannot call cudaMalloc: code inside a framework whose
caching allocator owns nearly all device memory (an allocation behind its back
can fail, and cudaFree synchronises the device), fitters that evaluate many
parameter points per second and cannot take that synchronisation in their
loop, and plugins handed only device pointers and a stream.  Its scratch is
one static device array shared by all calls, so two calls in a row with
different grids, bodies and neutrino types check that nothing carries over
from one call to the next.  Both paths build the same tables with the same
code, so their planes must be equal bit for bit.  This file is collected last
so that a run that stops at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

from cudaprob3_gb300 import _lib
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu

CODE = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def handle_path(cp, precision, cos, en, body, params, anti):
    with cp.CudaPropagatorSingle(0, len(cos), len(en), precision=precision) as p:
        p.setEnergyList(en)
        p.setCosineList(cos)
        p.setMNSMatrix(*params[:4])
        p.setNeutrinoMasses(*params[4:])
        p.setDensity(body.radii, body.rhos, body.ye)
        p.setProductionHeight(22.0)
        p.calculateProbabilities(cp.Antineutrino if anti else cp.Neutrino)
        return p.results().astype(np.float64)


def noalloc_path(torch, precision, cos, en, body, params, anti):
    lib = _lib.load()
    dc = torch.tensor(np.asarray(cos), dtype=torch.float64, device="cuda:0")
    de = torch.tensor(np.asarray(en), dtype=torch.float64, device="cuda:0")
    dt = torch.float32 if precision == "mixed" else torch.float64
    out = torch.full((9, len(cos), len(en)), -1.0, dtype=dt, device="cuda:0")
    r = np.ascontiguousarray(body.radii, dtype=np.float64)
    d = np.ascontiguousarray(body.rhos, dtype=np.float64)
    y = np.ascontiguousarray(body.ye, dtype=np.float64)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    rc = lib.cp3_propagate_noalloc(CODE[precision], 1 if anti else 0, ctypes.c_void_p(dc.data_ptr()), len(cos),
                                   ctypes.c_void_p(de.data_ptr()), len(en), dp(r), dp(d), dp(y), int(r.size),
                                   *[float(x) for x in params], 22.0, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.cp3_last_error().decode()
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_matches_handle_path_twice(gpu, precision):
    torch = pytest.importorskip("torch")
    calls = [
        (G.linspace(-1.0, 0.2, 300), G.logspace(0.1, 1000.0, 257), G.PREM_12, G.NOMINAL, False),
        (G.linspace(-1.0, 0.0, 1000), G.logspace(0.5, 100.0, 97), G.PREM_4,
         tuple(G.draw_parameter_sets(2, seed=4)[1]), True),
    ]
    for cos, en, body, params, anti in calls:
        got = noalloc_path(torch, precision, cos, en, body, params, anti)
        want = handle_path(gpu, precision, cos, en, body, params, anti)
        assert np.array_equal(got, want), "max |dP| %.3g" % np.abs(got - want).max()


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    lib = _lib.load()
    r = np.array(G.PREM_4.radii)
    d = np.array(G.PREM_4.rhos)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    args = [float(x) for x in G.NOMINAL] + [22.0]
    rc = lib.cp3_propagate_noalloc(1, 0, ctypes.c_void_p(16), 8193, ctypes.c_void_p(16), 16, dp(r), dp(d), None,
                                   int(r.size), *args, ctypes.c_void_p(16), None)
    assert rc == _lib.ERR_LIMIT and b"8192" in lib.cp3_last_error()
    r16 = np.linspace(0.0, 6371.0, 16)
    d16 = np.full(16, 4.0)
    rc = lib.cp3_propagate_noalloc(1, 0, ctypes.c_void_p(16), 16, ctypes.c_void_p(16), 16, dp(r16), dp(d16), None,
                                   16, *args, ctypes.c_void_p(16), None)
    assert rc == _lib.ERR_LIMIT and b"rows" in lib.cp3_last_error()
    # non-finite radii and densities are refused like cp3_set_density refuses them
    for bad_r, bad_d in ((np.inf, 4.0), (6371.0, np.inf), (np.nan, 4.0)):
        rb = r.copy()
        db = d.copy()
        rb[-1] = bad_r
        db[-1] = bad_d
        rc = lib.cp3_propagate_noalloc(1, 0, ctypes.c_void_p(16), 16, ctypes.c_void_p(16), 16, dp(rb), dp(db), None,
                                       int(rb.size), *args, ctypes.c_void_p(16), None)
        assert rc == _lib.ERR_ARGUMENT and b"finite" in lib.cp3_last_error()

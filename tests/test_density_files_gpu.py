"""The reference's density model files (example/models/PREM_{4,10,12,59}layer.dat,
copied into tests/golden/models/ by make_golden.py) read by this library's own
file loader -- cp3_set_density_from_file through the Python mirror, and the C++
class's setDensityFromFile -- against the reference's setDensityFromFile
(propagator.hpp:169-184) run on the same files (goldens file_*.npz).  Two
variants of the 12-layer file cover the read loop's edge cases: trailing blank
lines (skipped) and an outside-in copy with a text row after its eighth row
(the read stops there, so the eight rows above it form the body).

Tolerances: FP64 1e-11, mixed 1e-6 (max |dP| over the nine channels).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, load_golden
from cudaprob3_gb300 import grids as G

MODELS = os.path.join(GOLDEN, "models")
FILES = sorted(f for f in os.listdir(MODELS) if f.endswith(".dat"))
TOL = {"fp64": 1e-11, "mixed": 1e-6}


def test_every_model_file_has_a_golden():
    assert len(FILES) == 6
    for f in FILES:
        g = load_golden("file_" + f[:-4])
        # the rows stored with each golden are those the read loop takes
        r, d = G.read_density_file(os.path.join(MODELS, f))
        assert np.array_equal(r, g["radii"]) and np.array_equal(d, g["rhos"])


def test_read_loop_edge_cases():
    """Trailing blank lines are skipped; a text row ends the read, so the
    outside-in file whose ninth line is text yields its eight outermost rows."""
    full = load_golden("file_PREM_12layer")
    blank = load_golden("file_PREM_12layer_trailing_blank")
    text = load_golden("file_PREM_12layer_stops_at_text")
    assert np.array_equal(blank["radii"], full["radii"]) and np.array_equal(blank["probs"], full["probs"])
    assert np.array_equal(text["radii"], full["radii"][::-1][:8])
    assert np.isfinite(text["probs"]).all() and not np.array_equal(text["probs"], full["probs"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", FILES)
def test_file_loader_matches_reference(gpu, precision, name):
    g = load_golden("file_" + name[:-4])
    c, e = g["cosines"], g["energies"]
    with gpu.CudaPropagatorSingle(0, c.size, e.size, precision=precision) as p:
        p.setEnergyList(e)
        p.setCosineList(c)
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensityFromFile(os.path.join(MODELS, name))
        p.setProductionHeight(22.0)
        # the layer counts follow from the rows the loader read
        assert np.array_equal(p.maxlayers(), oracle.maxlayers(c, g["radii"]))
        p.calculateProbabilities(gpu.Neutrino)
        got = p.results().astype(np.float64)
    err = np.abs(got - g["probs"]).max()
    assert err <= TOL[precision], "%s %s: max|dP| = %.3g" % (name, precision, err)


@pytest.mark.gpu
def test_cpp_set_density_from_file(gpu):
    """tests/cpp/dropin_example.cpp (the reference example's usage: its six
    propagators read the body with setDensityFromFile) on every model file:
    the FP64 propagators against the reference's goldens, the float ones
    against the oracle on the float-rounded inputs."""
    from test_dropin_cpp import compile_example
    nc, ne = 37, 45
    per = nc + ne + nc * ne * 9
    kinds = ((1e-11, False), (1e-6, True), (1e-11, False), (1e-6, True), (1e-11, False), (1e-11, False))
    with tempfile.TemporaryDirectory() as d:
        exe = compile_example(d)
        for name in FILES:
            g = load_golden("file_" + name[:-4])
            out = os.path.join(d, "out.bin")
            r = subprocess.run([exe, out, os.path.join(MODELS, name)], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            raw = np.fromfile(out, dtype=np.float64)
            assert raw.size == len(kinds) * per
            for k, (tol, f32) in enumerate(kinds):
                blk = raw[k * per:(k + 1) * per]
                c, e = blk[:nc], blk[nc:nc + ne]
                got = blk[nc + ne:].reshape(nc, ne, 9).transpose(2, 0, 1)
                if not f32:
                    assert np.array_equal(c, g["cosines"]) and np.array_equal(e, g["energies"])
                    err = np.abs(got - g["probs"]).max()
                else:
                    cast = lambda x: np.asarray(x, dtype=np.float32).astype(np.float64)  # noqa: E731
                    params = tuple(float(cast(x)) for x in G.NOMINAL)
                    want = oracle.calculate(c, e, cast(g["radii"]), cast(g["rhos"]), params, float(cast(22.0)),
                                            False)
                    err = np.abs(got - want).max()
                assert err <= tol, "%s propagator %d: %.3g" % (name, k, err)

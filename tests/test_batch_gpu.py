"""Batched persistent kernel: every set against the oracle and against the
single-grid kernel, sequential launches equal to the graph launch, autotuner."""
import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu


def make_sets(n, seed):
    rng = np.random.default_rng(seed)
    nc = rng.integers(1, 97, size=n)
    ne = rng.integers(1, 130, size=n)
    nc[0], ne[0] = 1, 1
    params = G.draw_parameter_sets(n, seed=seed)
    scale = rng.uniform(0.97, 1.03, size=n)
    cos = [G.linspace(-1, 0.3, int(c)) if c > 1 else np.array([-0.4]) for c in nc]
    en = [G.logspace(0.5, 100.0, int(e)) if e > 1 else np.array([2.0]) for e in ne]
    return nc, ne, params, scale, cos, en


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-11)])
@pytest.mark.parametrize("anti", [False, True])
def test_batch_matches_oracle(gpu, precision, tol, anti):
    from cudaprob3_gb300.batch import BatchPropagator
    nc, ne, params, scale, cos, en = make_sets(12, seed=5)
    B = G.PREM_12
    with BatchPropagator(0, nc, ne, precision=precision) as b:
        b.set_grids(cos, en)
        b.set_parameters(params)
        b.set_density(B.radii, B.rhos, B.ye, scale)
        b.set_production_height(22.0)
        b.calculate(1 if anti else 0)
        flat = b.results()
        for s in range(len(nc)):
            got = b.set_result(flat, s).astype(np.float64)
            want = oracle.calculate(cos[s], en[s], B.radii, B.rho_eff() * scale[s], tuple(params[s]), 22.0, anti)
            assert np.abs(got - want).max() <= tol, "set %d" % s
        # the same work as two launches per set gives identical results
        b.calculate_sequential(1 if anti else 0)
        assert np.array_equal(b.results(), flat)
        # one prep launch per chunk (at most 8) and one propagate launch per
        # chunk that holds work items
        n = b.launch_count(1 if anti else 0)
        assert 2 <= n <= 16


def _prem59():
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "prem59.npz"))
    return G.Body(d["radii"], d["rhos"], d["ye"])


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-11)])
@pytest.mark.parametrize("body_name", ["prem4", "prem59"])
def test_batch_other_bodies(gpu, precision, tol, body_name):
    """5 layers (prep blocks of one warp, neighbours by shuffles) and 61
    layers (prep blocks of two warps, neighbours through shared memory)."""
    from cudaprob3_gb300.batch import BatchPropagator
    nc, ne, params, scale, cos, en = make_sets(6, seed=11)
    B = G.PREM_4 if body_name == "prem4" else _prem59()
    with BatchPropagator(0, nc, ne, precision=precision) as b:
        b.set_grids(cos, en)
        b.set_parameters(params)
        b.set_density(B.radii, B.rhos, B.ye, scale)
        b.set_production_height(22.0)
        b.calculate(0)
        te, groups, cchunk, _ = b.launch_shape()
        if body_name == "prem59" and precision == "fp64":
            # FP64 tables of 61 layers for a tile of 64 energies exceed shared
            # memory: the handle halves the tile
            assert te == 32
        flat = b.results()
        for s in range(len(nc)):
            got = b.set_result(flat, s).astype(np.float64)
            want = oracle.calculate(cos[s], en[s], B.radii, B.rho_eff() * scale[s], tuple(params[s]), 22.0, False)
            assert np.abs(got - want).max() <= tol, "set %d" % s


def test_batch_autotune_and_shapes(gpu):
    from cudaprob3_gb300.batch import BatchPropagator
    nc, ne, params, scale, cos, en = make_sets(20, seed=7)
    B = G.PREM_12
    with BatchPropagator(0, nc, ne, precision="mixed") as b:
        b.set_grids(cos, en)
        b.set_parameters(params)
        b.set_density(B.radii, B.rhos, B.ye, scale)
        b.set_production_height(22.0)
        b.calculate(0)
        ref = b.results()
        (te, g, cc), ms = b.autotune(0, reps=1)
        assert te in (32, 64, 128) and te * g <= 256 and ms > 0
        b.calculate(0)
        assert np.array_equal(b.results(), ref)
        for shape in ((32, 8, 8), (128, 2, 64), (64, 1, 16)):
            b.set_launch_shape(*shape)
            b.calculate(0)
            assert np.array_equal(b.results(), ref)


def test_batch_errors(gpu):
    from cudaprob3_gb300 import CP3Error
    from cudaprob3_gb300.batch import BatchPropagator
    with BatchPropagator(0, [3, 4], [5, 6]) as b:
        with pytest.raises(CP3Error, match="grids were not set"):
            b.calculate(0)
        b.set_grids([np.linspace(-1, 0, 3), np.linspace(-1, 0, 4)], [np.ones(5), np.ones(6)])
        with pytest.raises(CP3Error, match="parameters were not set"):
            b.calculate(0)
        with pytest.raises(CP3Error, match="unsupported launch shape"):
            b.set_launch_shape(48, 2, 8)
        # the body goes through the single-grid handle's checks (propagator.hpp:117-161)
        with pytest.raises(CP3Error, match="radii order messed up"):
            b.set_density([0.0, 3000.0, 2000.0], [1.0, 1.0, 1.0])
        with pytest.raises(CP3Error, match="must be finite"):
            b.set_density([0.0, np.inf], [1.0, 1.0])
        with pytest.raises(CP3Error, match="must be finite"):
            b.set_density([0.0, 6371.0], [1.0, -1.0])
        with pytest.raises(CP3Error, match="electron fractions"):
            b.set_density([0.0, 6371.0], [1.0, 1.0], [0.5, 1.5])
        with pytest.raises(CP3Error, match="more than 64 rows"):
            b.set_density(np.linspace(0.0, 6371.0, 65), np.ones(65))

"""Production-height distribution: probabilities averaged over heights with
weights, against the weighted average of the oracle's probabilities at each
height (the reference takes one height per calculation).

Tolerances (max |dP|): fp64 1e-11, mixed 1e-6.
"""
import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "mixed": 1e-6}


def make(cp, precision, c, e, body=G.PREM_12):
    p = cp.CudaPropagatorSingle(0, len(c), len(e), precision=precision)
    p.setEnergyList(e)
    p.setCosineList(c)
    p.setMNSMatrix(*G.NOMINAL[:4])
    p.setNeutrinoMasses(*G.NOMINAL[4:])
    p.setDensity(body.radii, body.rhos, body.ye)
    return p


def oracle_avg(c, e, heights, weights, anti, body=G.PREM_12):
    w = np.asarray(weights, float) / np.sum(weights)
    return sum(wk * oracle.calculate(c, e, body.radii, body.rho_eff(), G.NOMINAL, float(h), anti)
               for h, wk in zip(heights, w))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("anti", [False, True])
def test_height_average_vs_oracle(gpu, precision, anti):
    c = G.linspace(-1, 1, 61)  # downgoing (atmosphere only) and Earth-crossing
    e = G.logspace(0.1, 50, 77)
    heights = [5.0, 12.0, 18.0, 25.0, 40.0, 60.0]
    weights = [0.05, 0.2, 0.3, 0.25, 0.15, 0.05]
    with make(gpu, precision, c, e) as p:
        p.setProductionHeights(heights, weights)
        p.calculateProbabilities(gpu.Antineutrino if anti else gpu.Neutrino)
        got = p.results().astype(np.float64)
    want = oracle_avg(c, e, heights, weights, anti)
    assert np.abs(got - want).max() <= TOL[precision]
    # the average of unitary evolutions stays doubly stochastic
    s = got.reshape(3, 3, len(c), len(e))
    assert np.abs(s.sum(axis=0) - 1).max() <= 10 * TOL[precision]
    assert np.abs(s.sum(axis=1) - 1).max() <= 10 * TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_height_distribution_edge_cases(gpu, precision):
    c = G.linspace(-1, 0.5, 23)
    e = G.logspace(0.3, 20, 19)
    with make(gpu, precision, c, e, G.PREM_4) as p:
        p.setProductionHeight(22.0)
        p.calculateProbabilities(gpu.Neutrino)
        single = p.results()
        # one height is the single-height calculation
        p.setProductionHeights([22.0], [3.0])
        p.calculateProbabilities(gpu.Neutrino)
        assert np.array_equal(p.results(), single)
        # equal heights with any weights reproduce that height
        p.setProductionHeights([22.0, 22.0, 22.0], [1.0, 2.0, 0.5])
        p.calculateProbabilities(gpu.Neutrino)
        assert np.abs(p.results().astype(np.float64) - single).max() <= TOL[precision]
        # a zero weight removes its height
        p.setProductionHeights([22.0, 80.0], [1.0, 0.0])
        p.calculateProbabilities(gpu.Neutrino)
        assert np.abs(p.results().astype(np.float64) - single).max() <= TOL[precision]
        # setProductionHeight ends the distribution
        p.setProductionHeights([10.0, 30.0], [1.0, 1.0])
        p.calculateProbabilities(gpu.Neutrino)
        avg = p.results()
        want = oracle_avg(c, e, [10.0, 30.0], [1.0, 1.0], False, G.PREM_4)
        assert np.abs(avg.astype(np.float64) - want).max() <= TOL[precision]
        p.setProductionHeight(22.0)
        p.calculateProbabilities(gpu.Neutrino)
        assert np.array_equal(p.results(), single)
        # errors
        with pytest.raises(gpu.CP3Error, match="heights must be finite"):
            p.setProductionHeights([-1.0, 10.0], [1.0, 1.0])
        with pytest.raises(gpu.CP3Error, match="must not all be zero"):
            p.setProductionHeights([1.0, 10.0], [0.0, 0.0])
        with pytest.raises(gpu.CP3Error, match="CP3_MAX_HEIGHTS"):
            p.setProductionHeights(np.ones(65), np.ones(65))
        p.setProductionHeights([10.0, 30.0], [1.0, 1.0])
        p.setRateFlux(np.ones((3, len(c), len(e)), np.float32))
        p.setRateBins(np.zeros(len(c)), np.zeros(len(e)), 1, 1)
        with pytest.raises(gpu.CP3Error, match="height distribution"):
            p.calculateRates(gpu.Neutrino)
    with gpu.CudaPropagatorSingle(0, 3, 3) as p:
        with pytest.raises(gpu.CP3Error, match="must set cosine list before production height"):
            p.setProductionHeights([10.0, 20.0], [1.0, 1.0])

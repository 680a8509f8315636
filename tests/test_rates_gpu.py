"""Fused event rates: rate_b = sum_a flux_a P(a -> b) histogrammed inside the
propagation kernel, against the same sums formed from the oracle's
probabilities (numpy) and from the handle's own probability planes.

Tolerances, relative to the largest histogram entry: fp64 1e-12 against the
oracle; mixed 1e-6 against the oracle (|dP| <= 1e-7 per pair) and against its
own planes (FP32 sums of the short per-lane runs and a 5-level butterfly,
about 3e-7 of a bin at worst).
"""
import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu


def make(cp, precision, c, e, body=G.PREM_12):
    p = cp.CudaPropagatorSingle(0, len(c), len(e), precision=precision)
    p.setEnergyList(e)
    p.setCosineList(c)
    p.setMNSMatrix(*G.NOMINAL[:4])
    p.setNeutrinoMasses(*G.NOMINAL[4:])
    p.setDensity(body.radii, body.rhos, body.ye)
    p.setProductionHeight(22.0)
    return p


def hist_from_planes(P, flux, mask, cb, eb, ncb, neb):
    P = P.reshape(3, 3, *P.shape[1:]).astype(np.float64)
    f = flux.astype(np.float64) * np.array([(mask >> a) & 1 for a in range(3)], dtype=np.float64)[:, None, None]
    rate = np.einsum("acd,abcd->bcd", f, P)
    h = np.zeros((3, ncb, neb))
    keep = (cb[:, None] >= 0) & (eb[None, :] >= 0)
    ci, ei = np.nonzero(keep)
    for b in range(3):
        np.add.at(h[b], (cb[ci], eb[ei]), rate[b, ci, ei])
    return h


def contiguous_bins(n, nbins, lo_cut=0):
    b = (np.arange(n) * nbins) // n
    b[:lo_cut] = -1
    return b.astype(np.int32)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("anti", [False, True])
@pytest.mark.parametrize("mask", [3, 7])
def test_rates_monotone_bins_vs_oracle(gpu, precision, anti, mask):
    nc, ne = 150, 230
    c = G.linspace(-1, 0, nc)
    e = G.logspace(0.5, 100, ne)
    rng = np.random.default_rng(11 + mask)
    flux = rng.uniform(0.5, 2.0, size=(3, nc, ne)).astype(np.float32) * (e ** -2.7)[None, None, :].astype(np.float32)
    cb = contiguous_bins(nc, 12, lo_cut=3)
    eb = contiguous_bins(ne, 17)
    eb[-5:] = -1
    t = gpu.Antineutrino if anti else gpu.Neutrino
    with make(gpu, precision, c, e) as p:
        p.setRateFlux(flux, mask)
        p.setRateBins(cb, eb, 12, 17)
        got = p.calculateRates(t)
        p.calculateProbabilities(t)
        own = hist_from_planes(p.results(), flux, mask, cb, eb, 12, 17)
    P = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, anti)
    want = hist_from_planes(P, flux, mask, cb, eb, 12, 17)
    scale = np.abs(want).max()
    assert got.shape == (3, 12, 17)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.abs(got - want).max() <= tol * scale
    assert np.abs(got - own).max() <= (1e-13 if precision == "fp64" else 1e-6) * scale
    if mask == 3:
        # no tau flux: the tau-initial plane never enters
        assert np.abs(got.sum() - want.sum()) <= tol * np.abs(want).sum()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rates_scattered_bins(gpu, precision):
    """Non-monotone bin assignment (the per-lane fallback) and excluded nodes."""
    nc, ne = 97, 131
    c = G.linspace(-1, 1, nc)
    e = G.logspace(0.2, 300, ne)
    rng = np.random.default_rng(5)
    flux = rng.uniform(0.0, 1.0, size=(3, nc, ne)).astype(np.float32)
    cb = rng.integers(-1, 7, size=nc).astype(np.int32)
    eb = rng.integers(-1, 9, size=ne).astype(np.int32)
    with make(gpu, precision, c, e) as p:
        p.setRateFlux(flux)
        p.setRateBins(cb, eb, 7, 9)
        got = p.calculateRates(gpu.Neutrino)
    P = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, False)
    want = hist_from_planes(P, flux, 7, cb, eb, 7, 9)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.abs(got - want).max() <= tol * np.abs(want).max()


def test_rates_bench_shape_vs_planes(gpu):
    """1024 x 1024 fine grid into 40 x 50 bins, mixed: histogram of the fused
    path against the same sums over the handle's own planes."""
    n = 1024
    c = G.linspace(-1, 0, n)
    e = G.logspace(0.5, 100, n)
    flux = np.stack([0.5 * e ** -2.7, e ** -2.7, np.zeros(n)])[:, None, :].repeat(n, axis=1).astype(np.float32)
    cb = contiguous_bins(n, 40)
    eb = contiguous_bins(n, 50)
    with make(gpu, "mixed", c, e) as p:
        p.setRateFlux(flux, 3)
        p.setRateBins(cb, eb, 40, 50)
        got = p.calculateRates(gpu.Neutrino)
        again = p.calculateRates(gpu.Neutrino)
        p.calculateProbabilities(gpu.Neutrino)
        own = hist_from_planes(p.results(), flux, 3, cb, eb, 40, 50)
    scale = np.abs(own).max()
    assert np.abs(got - own).max() <= 1e-6 * scale
    assert np.abs(again - got).max() <= 1e-12 * scale  # re-zeroed between calculations


def test_rates_errors_and_empty(gpu):
    c = G.linspace(-1, 0, 8)
    e = G.logspace(1, 10, 9)
    with make(gpu, "mixed", c, e) as p:
        with pytest.raises(gpu.CP3Error, match="flux was not set"):
            p.calculateRates(gpu.Neutrino)
        p.setRateFlux(np.ones((3, 8, 9), np.float32))
        with pytest.raises(gpu.CP3Error, match="bins were not set"):
            p.calculateRates(gpu.Neutrino)
        with pytest.raises(gpu.CP3Error, match="out of range"):
            p.setRateBins(np.full(8, 3), np.zeros(9), 3, 1)
        with pytest.raises(gpu.CP3Error, match="mask"):
            p.setRateFlux(np.ones((3, 8, 9), np.float32), 9)
        p.setRateBins(np.zeros(8), np.zeros(9), 1, 1)
        h = p.calculateRates(gpu.Neutrino)
        # unit flux in every flavour: each final flavour receives sum_a P(a -> b),
        # and the three together receive 3 per node (unitarity)
        assert abs(h.sum() - 3 * 8 * 9) <= 1e-4
    with gpu.CudaPropagatorSingle(0, 0, 5, precision="mixed") as p:
        p.setEnergyList(G.logspace(1, 10, 5))
        p.setCosineList([])
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(G.PREM_4.radii, G.PREM_4.rhos)
        p.setProductionHeight(22.0)
        p.setRateFlux(np.ones((3, 0, 5), np.float32))
        p.setRateBins(np.zeros(0), np.zeros(5), 2, 2)
        assert not p.calculateRates(gpu.Neutrino).any()

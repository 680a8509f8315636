"""One propagation of a square grid, for profilers and quick timing.

    python -m cudaprob3_gb300.profile_case [--n 2048] [--precision mixed|fp64]
                                           [--repeat 1] [--anti]
                                           [--mode planes|rates|heights|gradient]

Grid: n cosines in [-1, 0] x n energies log-spaced over 0.1-1000 GeV on the
11-shell PREM body at the nominal parameters.  Modes: the nine planes; fused
event rates into 400 x 200 bins (flux E^-2.7, nu_e = nu_mu/2); planes
averaged over 8 production heights (10-45 km); gradient: evaluations of the
400 x 200 binned log-likelihood and its adjoint gradient (the n option does
not apply).  Prints the wall time of the repeated calculations.
"""
import argparse
import time

import numpy as np

import cudaprob3_gb300 as cp
from cudaprob3_gb300 import grids as G


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--anti", action="store_true")
    ap.add_argument("--mode", default="planes", choices=["planes", "rates", "heights", "gradient"])
    a = ap.parse_args()
    if a.mode == "gradient":
        from .loglik import binned_problem
        prob = binned_problem(device_id=0)
        L = prob.make(device_id=0, precision=a.precision)
        L.evaluate(prob.nominal, prob.body.rhos)
        t0 = time.perf_counter()
        for _ in range(a.repeat):
            L.evaluate(prob.nominal, prob.body.rhos)
        dt = time.perf_counter() - t0
        L.close()
        print("gradient precision=%s repeat=%d: %.3f ms per evaluation" % (a.precision, a.repeat, 1e3 * dt / a.repeat))
        return
    c = G.linspace(-1.0, 0.0, a.n)
    e = G.logspace(0.1, 1000.0, a.n)
    B = G.PREM_12
    with cp.CudaPropagatorSingle(0, a.n, a.n, precision=a.precision) as p:
        p.setEnergyList(e)
        p.setCosineList(c)
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(B.radii, B.rhos, B.ye)
        p.setProductionHeight(G.PRODUCTION_HEIGHT_KM)
        if a.mode == "heights":
            p.setProductionHeights(np.arange(10.0, 46.0, 5.0), [0.04, 0.10, 0.18, 0.22, 0.20, 0.14, 0.08, 0.04])
        if a.mode == "rates":
            phi = (e ** -2.7).astype(np.float32)
            flux = np.zeros((3, a.n, a.n), np.float32)
            flux[0] = 0.5 * phi[None, :]
            flux[1] = phi[None, :]
            p.setRateFlux(flux, 3)
            p.setRateBins((np.arange(a.n) * 400) // a.n, (np.arange(a.n) * 200) // a.n, 400, 200)
        t = cp.Antineutrino if a.anti else cp.Neutrino
        t0 = time.perf_counter()
        for _ in range(a.repeat):
            if a.mode == "rates":
                p.calculateRates(t)
            else:
                p.calculateProbabilities(t)
        dt = time.perf_counter() - t0
        print("n=%d precision=%s mode=%s repeat=%d: %.3f ms per calculation" % (a.n, a.precision, a.mode, a.repeat,
                                                                                1e3 * dt / a.repeat))


if __name__ == "__main__":
    main()

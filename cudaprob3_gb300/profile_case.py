"""One propagation of a square grid, for profilers and quick timing.

    python -m cudaprob3_gb300.profile_case [--n 2048] [--precision mixed|fp64]
                                           [--repeat 1] [--anti]

Grid: n cosines in [-1, 0] x n energies log-spaced over 0.1-1000 GeV on the
11-shell PREM body at the nominal parameters.  Prints the wall time of the
repeated calculations.
"""
import argparse
import time

import cudaprob3_gb300 as cp
from cudaprob3_gb300 import grids as G


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--anti", action="store_true")
    a = ap.parse_args()
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
        t = cp.Antineutrino if a.anti else cp.Neutrino
        t0 = time.perf_counter()
        for _ in range(a.repeat):
            p.calculateProbabilities(t)
        dt = time.perf_counter() - t0
        print("n=%d precision=%s repeat=%d: %.3f ms per calculation" % (a.n, a.precision, a.repeat,
                                                                        1e3 * dt / a.repeat))


if __name__ == "__main__":
    main()

"""Grids, bodies and parameter points used by the examples, tests and bench.

* ``linspace`` / ``logspace`` restate the example driver's grid builders
  (example/main.cpp:32-49 and 51-69): the step is accumulated, the end points
  are exact, and the log grid exponentiates an accumulated log step.
* ``PREM_4`` is the 4-shell body of example/models/PREM_4layer.dat; ``PREM_12``
  is the 11-shell body of the 12-row table (one inert radius-0 row).
* Electron fractions are native here (``ye``); the reference has none and
  multiplies every density by 0.5 (constants.hpp:40, physics.hpp:651).
"""
import math

import numpy as np


def linspace(lo, hi, n):
    """example/main.cpp:32-49 (accumulated step, exact last point)."""
    if n == 0:
        raise ValueError("div == 0")
    out = np.zeros(n, dtype=np.float64)
    step = (hi - lo) / float(n - 1) if n > 1 else 0.0
    ee = lo
    for i in range(n - 1):
        out[i] = ee
        ee += step
    out[n - 1] = hi
    return out


def logspace(lo, hi, n):
    """example/main.cpp:51-69 (exp of an accumulated log step, exact ends)."""
    if n == 0:
        raise ValueError("div == 0")
    out = np.zeros(n, dtype=np.float64)
    llo, lhi = math.log(lo), math.log(hi)
    step = (lhi - llo) / float(n - 1) if n > 1 else 0.0
    out[0] = lo
    ee = llo + step
    for i in range(1, n - 1):
        out[i] = math.exp(ee)
        ee += step
    out[n - 1] = hi
    return out


class Body:
    """Piecewise-constant sphere in the reference's file layout.

    ``radii`` ascending with a first row at radius 0 (propagator.hpp:163-168);
    ``rhos[i]`` is the density between ``radii[i-1]`` (exclusive) and
    ``radii[i]`` (inclusive); ``ye`` the electron fraction of that shell.
    """

    def __init__(self, radii, rhos, ye):
        self.radii = np.asarray(radii, dtype=np.float64)
        self.rhos = np.asarray(rhos, dtype=np.float64)
        self.ye = np.asarray(ye, dtype=np.float64)
        if not (self.radii.shape == self.rhos.shape == self.ye.shape):
            raise ValueError("radii, rhos and ye differ in length")

    def rho_eff(self):
        """Density that makes the reference's fixed 0.5 reproduce rho*ye."""
        return (self.rhos * self.ye) / 0.5

    def scaled(self, s):
        return Body(self.radii, self.rhos * s, self.ye)


YE_CORE = 0.468
YE_MANTLE = 0.497

# example/models/PREM_4layer.dat with the core/mantle electron fractions.
PREM_4 = Body([0.0, 1220.0, 3480.0, 5701.0, 6371.0],
              [13.0, 13.0, 11.3, 5.0, 3.3],
              [YE_CORE, YE_CORE, YE_CORE, YE_MANTLE, YE_MANTLE])

# 11 shells plus the inert radius-0 row (12 rows in the reference's format).
PREM_12 = Body([0.0, 1221.5, 3480.0, 3630.0, 5701.0, 5771.0, 5971.0, 6151.0, 6346.6,
                6356.0, 6368.0, 6371.0],
               [13.0, 13.0, 11.3, 5.5, 5.0, 4.4, 4.0, 3.5, 3.4, 3.0, 2.6, 1.02],
               [YE_CORE, YE_CORE, YE_CORE] + [YE_MANTLE] * 9)

# Nominal oscillation point: theta12, theta13, theta23, dCP [rad], dm21^2, dm32^2 [eV^2].
NOMINAL = (0.5837, 0.1496, 0.8587, 3.86, 7.42e-5, 2.51e-3)
PRODUCTION_HEIGHT_KM = 22.0

# Widths of the Gaussian parameter draws around NOMINAL (theta, dCP, dm21, dm32).
SIGMA = (0.02, 0.02, 0.02, 1.0, 2e-6, 5e-5)


def draw_parameter_sets(n, seed=0):
    """n Gaussian parameter points around NOMINAL, drawn in the fixed order
    theta12, theta13, theta23, dCP, dm21, dm32 (normals) then a uniform bit for
    the sign of dm32 per set."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, 6))
    sign = rng.integers(0, 2, size=n)
    out = np.empty((n, 6), dtype=np.float64)
    for k in range(6):
        out[:, k] = NOMINAL[k] + SIGMA[k] * z[:, k]
    out[:, 5] = np.where(sign == 1, -out[:, 5], out[:, 5])
    return out


def read_density_file(path):
    """Two whitespace-separated columns (radius km, density g/cm^3), read until
    the first pair that does not parse (propagator.hpp:169-184)."""
    radii, rhos = [], []
    with open(path) as f:
        toks = f.read().split()
    for i in range(0, len(toks) - 1, 2):
        try:
            r, d = float(toks[i]), float(toks[i + 1])
        except ValueError:
            break
        radii.append(r)
        rhos.append(d)
    return np.array(radii), np.array(rhos)

"""Binned Poisson log-likelihood and its adjoint gradient (C ABI: cp3_loglik_*).

Bin (c, e) expects lambda = norm * (flux_e[e] P(e->mu) + flux_mu[e] P(mu->mu))
events; LL = sum n ln(lambda) - lambda.  ``evaluate`` returns LL and the
gradient with respect to (theta12, theta13, theta23, dcp, dm12sq, dm23sq,
rho_row_0 .. rho_row_{n-1}).

``binned_problem`` builds the 400 cosine x 200 energy workload: bin centres
uniform in cos [-1, 0] and log-uniform in E over 0.5-100 GeV, a power-law flux
E^-2.7 for nu_mu and half of it for nu_e, a normalisation giving 1e6 expected
events at the nominal point, and Poisson counts (seed 1) drawn at a perturbed
parameter point with this library's FP64 propagator.
"""
import ctypes

import numpy as np

from . import _lib
from . import grids as G
from ._lib import check

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}
PARAM_NAMES = ("theta12", "theta13", "theta23", "dcp", "dm12sq", "dm23sq")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class LogLikelihood:
    def __init__(self, device_id, n_cosines, n_energies, precision="fp64"):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        self.n_cosines, self.n_energies = int(n_cosines), int(n_energies)
        self.n_rows = 0
        check(self._lib.cp3_loglik_create(ctypes.byref(self._h), int(device_id), _PRECISIONS[precision],
                                          self.n_cosines, self.n_energies))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cp3_loglik_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_bins(self, cosines, energies):
        c = np.ascontiguousarray(cosines, dtype=np.float64)
        e = np.ascontiguousarray(energies, dtype=np.float64)
        check(self._lib.cp3_loglik_set_bins(self._h, _dp(c), _dp(e)))

    def set_body(self, radii, ye=None):
        r = np.ascontiguousarray(radii, dtype=np.float64)
        y = None if ye is None else np.ascontiguousarray(ye, dtype=np.float64)
        check(self._lib.cp3_loglik_set_body(self._h, _dp(r), None if y is None else _dp(y), int(r.size)))
        self.n_rows = int(r.size)
        # argument buffers of evaluate, with their ctypes pointers made once:
        # building the pointers and arrays on every call costs about 7 us on
        # the GPU machine's host, more than a tenth of a mixed evaluation
        self._p = np.zeros(6)
        self._r = np.zeros(self.n_rows)
        self._g = np.zeros(6 + self.n_rows)
        self._ll = ctypes.c_double()
        self._args = (_dp(self._p), _dp(self._r), ctypes.byref(self._ll), _dp(self._g))

    def set_production_height(self, km):
        check(self._lib.cp3_loglik_set_production_height(self._h, float(km)))

    def set_flux(self, flux_e, flux_mu, norm):
        fe = np.ascontiguousarray(flux_e, dtype=np.float64)
        fm = np.ascontiguousarray(flux_mu, dtype=np.float64)
        check(self._lib.cp3_loglik_set_flux(self._h, _dp(fe), _dp(fm), float(norm)))

    def set_observed(self, counts):
        n = np.ascontiguousarray(counts, dtype=np.float64).reshape(self.n_cosines, self.n_energies)
        check(self._lib.cp3_loglik_set_observed(self._h, _dp(n)))

    def evaluate(self, params, rhos, ntype=0):
        """(LL, gradient) at the 6 oscillation parameters and the row
        densities (one per row of the body); the gradient is a new array."""
        if not self.n_rows:  # no body yet: the C call reports what is missing
            p = np.ascontiguousarray(params, dtype=np.float64)
            r = np.ascontiguousarray(rhos, dtype=np.float64)
            ll = ctypes.c_double()
            grad = np.empty(6, dtype=np.float64)
            check(self._lib.cp3_loglik_evaluate(self._h, int(ntype), _dp(p), _dp(r), ctypes.byref(ll), _dp(grad)))
            return ll.value, grad
        self._p[:] = params  # raises unless there are 6 parameters and n_rows densities
        self._r[:] = rhos
        check(self._lib.cp3_loglik_evaluate(self._h, int(ntype), *self._args))
        return self._ll.value, self._g.copy()

    def set_kernel_timing(self, enable):
        """CUDA events around the evaluation's kernels (the graph is captured
        again with or without them)."""
        check(self._lib.cp3_loglik_set_kernel_timing(self._h, 1 if enable else 0))

    def last_kernel_ms(self):
        """(prep, pair, layer) kernel durations of the last timed evaluation."""
        t = [ctypes.c_float() for _ in range(3)]
        check(self._lib.cp3_loglik_last_kernel_ms(self._h, *[ctypes.byref(x) for x in t]))
        return tuple(x.value for x in t)

    def io_bytes(self):
        """(host-to-device, device-to-host) bytes of one evaluation."""
        up, down = ctypes.c_longlong(), ctypes.c_longlong()
        check(self._lib.cp3_loglik_io_bytes(self._h, ctypes.byref(up), ctypes.byref(down)))
        return up.value, down.value


class BinnedProblem:
    """The inputs of a binned fit (see the module docstring)."""

    def __init__(self, cosines, energies, body, flux_e, flux_mu, norm, counts, nominal, observed_at, height=22.0):
        self.cosines, self.energies, self.body = cosines, energies, body
        self.flux_e, self.flux_mu, self.norm = flux_e, flux_mu, norm
        self.counts, self.nominal, self.observed_at, self.height = counts, nominal, observed_at, height

    def expected(self, pem, pmm):
        """lambda[c][e] from P(e->mu) and P(mu->mu) arrays [n_cos][n_en]."""
        return self.norm * (self.flux_e[None, :] * pem + self.flux_mu[None, :] * pmm)

    def loglik(self, pem, pmm):
        lam = self.expected(pem, pmm)
        return float(np.sum(self.counts * np.log(lam) - lam))

    def loglik_abs_sum(self, planes):
        """sum_b |n_b ln(lambda_b)| + lambda_b for the nine planes [9][nc][ne]:
        the scale of the rounding error of one log-likelihood evaluation."""
        lam = self.expected(planes[1], planes[4])
        return float(np.sum(np.abs(self.counts * np.log(lam)) + lam))

    def make(self, device_id=0, precision="fp64"):
        L = LogLikelihood(device_id, self.cosines.size, self.energies.size, precision)
        L.set_bins(self.cosines, self.energies)
        L.set_body(self.body.radii, self.body.ye)
        L.set_production_height(self.height)
        L.set_flux(self.flux_e, self.flux_mu, self.norm)
        L.set_observed(self.counts)
        return L


def _probabilities(cos, en, body, params, rhos, device_id, height):
    from .propagator import CudaPropagatorSingle, Neutrino
    with CudaPropagatorSingle(device_id, cos.size, en.size, precision="fp64") as p:
        p.setEnergyList(en)
        p.setCosineList(cos)
        p.setMNSMatrix(*params[:4])
        p.setNeutrinoMasses(*params[4:])
        p.setDensity(body.radii, rhos, body.ye)
        p.setProductionHeight(height)
        p.calculateProbabilities(Neutrino)
        r = p.results()
    return r[1], r[4]  # P(e -> mu), P(mu -> mu)


def binned_problem(n_cos=400, n_en=200, device_id=0, seed=1, total=1.0e6, body=None):
    cos = -1.0 + (np.arange(n_cos) + 0.5) / n_cos
    edges = np.exp(np.linspace(np.log(0.5), np.log(100.0), n_en + 1))
    en = np.sqrt(edges[:-1] * edges[1:])
    body = G.PREM_12 if body is None else body
    flux_mu = en ** -2.7
    flux_e = 0.5 * flux_mu
    nominal = np.array(G.NOMINAL, dtype=np.float64)
    # observed at a shifted point: +1 sigma in theta23, dcp and dm32
    observed_at = nominal + np.array([0.0, 0.0, G.SIGMA[2], G.SIGMA[3], 0.0, G.SIGMA[5]])
    pem0, pmm0 = _probabilities(cos, en, body, nominal, body.rhos, device_id, 22.0)
    norm = total / float(np.sum(flux_e[None, :] * pem0 + flux_mu[None, :] * pmm0))
    pem, pmm = _probabilities(cos, en, body, observed_at, body.rhos, device_id, 22.0)
    lam = norm * (flux_e[None, :] * pem + flux_mu[None, :] * pmm)
    counts = np.random.default_rng(seed).poisson(lam).astype(np.float64)
    return BinnedProblem(cos, en, body, flux_e, flux_mu, norm, counts, nominal, observed_at)

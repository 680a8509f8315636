"""Python mirror of the reference's propagator interface.

``CudaPropagatorSingle`` keeps the names, argument meaning and error
behaviour of cudaprob3::CudaPropagatorSingle<FLOAT_T> (cudapropagator.cuh:39-251)
and its base cudaprob3::Propagator<FLOAT_T> (propagator.hpp:43-337); every call
goes through the C ABI of libcudaprob3_gb300.so.  ``precision`` plays the role
of FLOAT_T: "fp64" is the plain FP64 method (double results), "mixed" the
double-float eigen-solve / 32-bit bulk method (float results).
"""
import ctypes
import enum

import numpy as np

from . import _lib
from ._lib import CP3Error, check


class NeutrinoType(enum.IntEnum):
    """types.hpp:29"""
    Neutrino = 0
    Antineutrino = 1


class ProbType(enum.IntEnum):
    """types.hpp:23-27: index = in*3 + out, x_y is P(x -> y)."""
    e_e = 0
    e_m = 1
    e_t = 2
    m_e = 3
    m_m = 4
    m_t = 5
    t_e = 6
    t_m = 7
    t_t = 8


Neutrino = NeutrinoType.Neutrino
Antineutrino = NeutrinoType.Antineutrino

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "double": _lib.PRECISION_FP64,
               "mixed": _lib.PRECISION_MIXED, "float": _lib.PRECISION_MIXED}


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def device_count():
    return int(_lib.load().cp3_device_count())


class CudaPropagatorSingle:
    """Single-GPU propagator: CudaPropagatorSingle(id, n_cosines, n_energies)."""

    def __init__(self, device_id, n_cosines, n_energies=None, precision="fp64"):
        if n_energies is None:  # CudaPropagatorSingle(n_cosines, n_energies) on device 0
            device_id, n_cosines, n_energies = 0, device_id, n_cosines
        if precision not in _PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(_PRECISIONS))
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.cp3_create(ctypes.byref(self._h), int(device_id), int(n_cosines), int(n_energies),
                                   _PRECISIONS[precision]))
        self.device_id = int(device_id)
        self.n_cosines = int(n_cosines)
        self.n_energies = int(n_energies)
        self.precision = "fp64" if _PRECISIONS[precision] == _lib.PRECISION_FP64 else "mixed"
        self.dtype = np.float64 if self.precision == "fp64" else np.float32

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cp3_destroy(self._h)
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

    # -- Propagator<FLOAT_T> setters (propagator.hpp:117-286) ------------------
    def setEnergyList(self, energies):
        e = np.ascontiguousarray(energies, dtype=np.float64)
        check(self._lib.cp3_set_energy_list(self._h, _dptr(e), int(e.size)))

    def setCosineList(self, cosines):
        c = np.ascontiguousarray(cosines, dtype=np.float64)
        check(self._lib.cp3_set_cosine_list(self._h, _dptr(c), int(c.size)))

    def setMNSMatrix(self, theta12, theta13, theta23, dcp):
        check(self._lib.cp3_set_mns_matrix(self._h, float(theta12), float(theta13), float(theta23), float(dcp)))

    def setNeutrinoMasses(self, dm12sq, dm23sq):
        check(self._lib.cp3_set_neutrino_masses(self._h, float(dm12sq), float(dm23sq)))

    def setDensity(self, radii, rhos, ye=None):
        """Shell table as in propagator.hpp:117-161; ``ye`` (electron fraction
        per row) defaults to the reference's fixed 0.5."""
        r = np.ascontiguousarray(radii, dtype=np.float64)
        d = np.ascontiguousarray(rhos, dtype=np.float64)
        if r.size != d.size:
            raise CP3Error(_lib.ERR_ARGUMENT, "setDensity : rhos.size() != radii.size()")
        y = None if ye is None else np.ascontiguousarray(ye, dtype=np.float64)
        if y is not None and y.size != r.size:
            raise CP3Error(_lib.ERR_ARGUMENT, "setDensity : ye.size() != radii.size()")
        check(self._lib.cp3_set_density(self._h, _dptr(r), _dptr(d), None if y is None else _dptr(y),
                                        int(r.size)))

    def setDensityFromFile(self, filename):
        check(self._lib.cp3_set_density_from_file(self._h, str(filename).encode()))

    def setProductionHeight(self, height_km):
        check(self._lib.cp3_set_production_height(self._h, float(height_km)))

    # -- calculation (cudapropagator.cuh:162-235) -----------------------------
    def setProductionHeights(self, heights_km, weights):
        """Average the probabilities over production heights (km) with the
        given weights (normalised); no reference counterpart (the reference
        takes one height).  setProductionHeight ends the distribution."""
        h = np.ascontiguousarray(heights_km, dtype=np.float64)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if h.shape != w.shape or h.ndim != 1:
            raise ValueError("one weight per height")
        check(self._lib.cp3_set_production_heights(self._h, _dptr(h), _dptr(w), int(h.size)))

    def calculateProbabilities(self, ntype):
        check(self._lib.cp3_calculate_probabilities(self._h, int(ntype)))

    def calculateProbabilitiesAsync(self, ntype):
        check(self._lib.cp3_calculate_probabilities_async(self._h, int(ntype)))

    def waitForCompletion(self):
        check(self._lib.cp3_wait_for_completion(self._h))

    def getProbability(self, index_cosine, index_energy, t):
        out = ctypes.c_double()
        check(self._lib.cp3_get_probability(self._h, int(index_cosine), int(index_energy), int(t),
                                            ctypes.byref(out)))
        return out.value

    # -- bulk access (no reference counterpart) -------------------------------
    def result_bytes(self):
        n = ctypes.c_size_t()
        check(self._lib.cp3_result_bytes(self._h, ctypes.byref(n)))
        return n.value

    def result_device_ptr(self):
        p = ctypes.c_void_p()
        check(self._lib.cp3_result_device_ptr(self._h, ctypes.byref(p)))
        return p.value

    def results(self, out=None):
        """All probabilities as [9][n_cosines][n_energies] (plane in*3+out)."""
        shape = (9, self.n_cosines, self.n_energies)
        if out is None:
            out = np.empty(shape, dtype=self.dtype)
        if out.dtype != self.dtype or out.shape != shape or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous %s array of shape %s" % (self.dtype, shape))
        check(self._lib.cp3_copy_results_to_host(self._h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def copy_results_to(self, host_ptr, nbytes):
        check(self._lib.cp3_copy_results_to_host(self._h, ctypes.c_void_p(host_ptr), int(nbytes)))

    def set_result_buffer(self, device_ptr, nbytes):
        check(self._lib.cp3_set_result_buffer(self._h, ctypes.c_void_p(device_ptr), int(nbytes)))

    def set_host_result_buffer(self, host_ptr, nbytes):
        """Zero-copy host results into page-locked memory at `host_ptr`
        (cudaHostAlloc / cudaHostRegister, e.g. a pinned torch tensor); 0
        returns to the device buffer.  Pageable memory raises CP3Error."""
        check(self._lib.cp3_set_host_result_buffer(self._h, ctypes.c_void_p(host_ptr), int(nbytes)))

    # ---- fused event rates (no reference counterpart; include/cudaprob3_gb300.h)
    def setRateFlux(self, flux, flavour_mask=7):
        """Per-(cosine, energy) weights of the initial flavours e, mu, tau:
        array [3][n_cosines][n_energies] (float32; planes whose bit is clear
        in `flavour_mask` are ignored), copied to the device."""
        f = np.ascontiguousarray(flux, dtype=np.float32)
        if f.shape != (3, self.n_cosines, self.n_energies):
            raise ValueError("flux must have shape (3, n_cosines, n_energies)")
        self._flux_host = f
        check(self._lib.cp3_set_rate_flux(self._h, f.ctypes.data_as(ctypes.c_void_p), int(flavour_mask), 0))

    def set_rate_flux_device(self, device_ptr, flavour_mask=7):
        """Flux already on the device (caller-owned [3][n_cos][n_en] float32)."""
        check(self._lib.cp3_set_rate_flux(self._h, ctypes.c_void_p(device_ptr), int(flavour_mask), 1))

    def setRateBins(self, cos_bin, en_bin, n_cos_bins, n_en_bins):
        """Histogram bin of every cosine and energy node (-1 leaves it out)."""
        cb = np.ascontiguousarray(cos_bin, dtype=np.int32)
        eb = np.ascontiguousarray(en_bin, dtype=np.int32)
        if cb.shape != (self.n_cosines,) or eb.shape != (self.n_energies,):
            raise ValueError("one bin index per cosine and per energy node")
        check(self._lib.cp3_set_rate_bins(self._h, cb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          eb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          int(n_cos_bins), int(n_en_bins)))
        self._rate_shape = (3, int(n_cos_bins), int(n_en_bins))

    def calculateRatesAsync(self, ntype):
        check(self._lib.cp3_calculate_rates_async(self._h, int(ntype)))

    def calculateRates(self, ntype, out=None):
        """Propagate and histogram rate_b = sum_a flux_a P(a -> b); returns the
        FP64 histograms [3][n_cos_bins][n_en_bins] (final flavour first)."""
        check(self._lib.cp3_calculate_rates(self._h, int(ntype)))
        return self.rates(out)

    def rates(self, out=None):
        if out is None:
            out = np.empty(self._rate_shape, dtype=np.float64)
        check(self._lib.cp3_get_rates(self._h, _dptr(out), out.size))
        return out

    def rates_device_ptr(self):
        p = ctypes.c_void_p()
        check(self._lib.cp3_rates_device_ptr(self._h, ctypes.byref(p)))
        return p.value

    def set_host_completion(self, enable=True):
        """With a host result buffer: the kernel stores the four planes of the
        2x2 flavour block and waitForCompletion derives the other five on the
        host cores (4/9 of the bytes over the host link)."""
        check(self._lib.cp3_set_host_completion(self._h, 1 if enable else 0))

    def set_stream(self, stream_handle):
        check(self._lib.cp3_set_stream(self._h, ctypes.c_void_p(stream_handle)))

    def maxlayers(self):
        out = np.empty(self.n_cosines, dtype=np.int32)
        check(self._lib.cp3_get_maxlayers(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          self.n_cosines))
        return out

    def set_kernel_timing(self, enable=True):
        check(self._lib.cp3_set_kernel_timing(self._h, 1 if enable else 0))

    def last_kernel_ms(self):
        """(prep_ms, propagate_ms) of the last timed calculation."""
        a, b = ctypes.c_float(), ctypes.c_float()
        check(self._lib.cp3_last_kernel_ms(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_launch_shape(self, te, groups, cchunk):
        check(self._lib.cp3_set_launch_shape(self._h, int(te), int(groups), int(cchunk)))

    def launch_shape(self):
        v = [ctypes.c_int() for _ in range(3)]
        check(self._lib.cp3_get_launch_shape(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def autotune(self, ntype=0, reps=2):
        """Time every supported launch shape on this grid; keep the fastest."""
        te, g, cc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_float()
        check(self._lib.cp3_autotune(self._h, int(ntype), int(reps), ctypes.byref(te), ctypes.byref(g),
                                     ctypes.byref(cc), ctypes.byref(ms)))
        return (te.value, g.value, cc.value), ms.value

    def last_launch_count(self):
        n = ctypes.c_int()
        check(self._lib.cp3_last_launch_count(self._h, ctypes.byref(n)))
        return n.value

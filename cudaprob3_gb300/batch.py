"""Batched propagation of many parameter sets (C ABI: cp3_batch_*).

Each set s has its own oscillation parameters, density scale and grid of
n_cosines[s] x n_energies[s] pairs; its probabilities are the reference's
[9][n_cosines[s]][n_energies[s]] planes.  One calculation is one CUDA-graph
launch (counter reset, batched FP64 precompute, persistent propagate kernel).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class BatchPropagator:
    def __init__(self, device_id, n_cosines, n_energies, precision="mixed"):
        self._lib = _lib.load()
        self.n_cosines = np.ascontiguousarray(n_cosines, dtype=np.int32)
        self.n_energies = np.ascontiguousarray(n_energies, dtype=np.int32)
        if self.n_cosines.shape != self.n_energies.shape:
            raise ValueError("n_cosines and n_energies differ in length")
        self.n_sets = int(self.n_cosines.size)
        self.precision = precision
        self.dtype = np.float32 if precision == "mixed" else np.float64
        self._h = ctypes.c_void_p()
        check(self._lib.cp3_batch_create(ctypes.byref(self._h), int(device_id), _PRECISIONS[precision],
                                         self.n_sets, _ip(self.n_cosines), _ip(self.n_energies)))
        off = np.empty(self.n_sets + 1, dtype=np.int64)
        check(self._lib.cp3_batch_result_offsets(self._h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        self.offsets = off

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cp3_batch_destroy(self._h)
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

    @property
    def total_pairs(self):
        return int(np.sum(self.n_cosines.astype(np.int64) * self.n_energies))

    def set_grids(self, cosines, energies):
        """Lists of per-set cosine and energy arrays (or pre-concatenated arrays)."""
        c = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in cosines])
                                 if isinstance(cosines, (list, tuple)) else cosines, dtype=np.float64)
        e = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in energies])
                                 if isinstance(energies, (list, tuple)) else energies, dtype=np.float64)
        if c.size != int(self.n_cosines.sum()) or e.size != int(self.n_energies.sum()):
            raise ValueError("grid sizes do not match the sets")
        check(self._lib.cp3_batch_set_grids(self._h, _dp(c), _dp(e)))

    def set_parameters(self, params):
        """params: [n_sets, 6] = theta12, theta13, theta23, dcp, dm12sq, dm23sq."""
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(self.n_sets, 6)
        check(self._lib.cp3_batch_set_parameters(self._h, _dp(p)))

    def set_density(self, radii, rhos, ye=None, scale=None):
        r = np.ascontiguousarray(radii, dtype=np.float64)
        d = np.ascontiguousarray(rhos, dtype=np.float64)
        y = None if ye is None else np.ascontiguousarray(ye, dtype=np.float64)
        s = None if scale is None else np.ascontiguousarray(scale, dtype=np.float64)
        check(self._lib.cp3_batch_set_density(self._h, _dp(r), _dp(d), None if y is None else _dp(y), int(r.size),
                                              None if s is None else _dp(s)))

    def set_production_height(self, km):
        check(self._lib.cp3_batch_set_production_height(self._h, float(km)))

    def set_stream(self, handle):
        check(self._lib.cp3_batch_set_stream(self._h, ctypes.c_void_p(handle)))

    def set_launch_shape(self, te, groups, cchunk):
        check(self._lib.cp3_batch_set_launch_shape(self._h, int(te), int(groups), int(cchunk)))

    def launch_shape(self):
        v = [ctypes.c_int() for _ in range(4)]
        check(self._lib.cp3_batch_get_launch_shape(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def autotune(self, ntype=0, reps=2):
        te, g, cc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_float()
        check(self._lib.cp3_batch_autotune(self._h, int(ntype), int(reps), ctypes.byref(te), ctypes.byref(g),
                                           ctypes.byref(cc), ctypes.byref(ms)))
        return (te.value, g.value, cc.value), ms.value

    def calculate(self, ntype=0):
        check(self._lib.cp3_batch_calculate(self._h, int(ntype)))

    def calculate_async(self, ntype=0):
        check(self._lib.cp3_batch_calculate_async(self._h, int(ntype)))

    def wait(self):
        check(self._lib.cp3_batch_wait(self._h))

    def calculate_sequential(self, ntype=0):
        check(self._lib.cp3_batch_calculate_sequential(self._h, int(ntype)))

    def last_ms(self):
        ms = ctypes.c_float()
        check(self._lib.cp3_batch_last_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def launch_count(self, ntype=0):
        """Kernels one calculate() launches (prep and propagate of every chunk)."""
        n = ctypes.c_int()
        check(self._lib.cp3_batch_launch_count(self._h, int(ntype), ctypes.byref(n)))
        return n.value

    def result_device_ptr(self):
        p = ctypes.c_void_p()
        check(self._lib.cp3_batch_result_device_ptr(self._h, ctypes.byref(p)))
        return p.value

    def maxlayers(self):
        out = np.empty(int(self.n_cosines.sum()), dtype=np.int32)
        check(self._lib.cp3_batch_get_maxlayers(self._h, _ip(out), ctypes.c_longlong(out.size)))
        return out

    def results(self):
        """All sets' planes as one flat array (split with ``offsets``)."""
        out = np.empty(int(self.offsets[-1]), dtype=self.dtype)
        check(self._lib.cp3_batch_copy_results_to_host(self._h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def set_result(self, flat, s):
        a, b = int(self.offsets[s]), int(self.offsets[s + 1])
        return flat[a:b].reshape(9, int(self.n_cosines[s]), int(self.n_energies[s]))

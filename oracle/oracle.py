"""ctypes front end of the oracle libraries (test infrastructure only)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libcp3ref.so")
_lib = None
_ref = None


def build(ref_dir="/root/reference"):
    """Compile liboracle.so (and oracle/_ref when the reference sources exist)."""
    env = dict(os.environ, REF_DIR=ref_dir)
    subprocess.run(["make", "-s", "-C", _HERE], check=True, env=env)


def _arch_ok(path):
    """True when the shared object at ``path`` loads on this machine."""
    try:
        ctypes.CDLL(path)
        return True
    except OSError:
        return False


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) or not _arch_ok(_LIB):
            build()
        _lib = ctypes.CDLL(_LIB)
        for sfx, ct in (("_f64", ctypes.c_double), ("_f32", ctypes.c_float)):
            f = getattr(_lib, "oracle_calculate" + sfx)
            P = ctypes.POINTER(ct)
            f.argtypes = [ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P, P,
                          ct, ct, ct, ct, ct, ct, ct, ctypes.c_int, ctypes.c_int, P]
            f.restype = ctypes.c_int
            g = getattr(_lib, "oracle_maxlayers" + sfx)
            g.argtypes = [ctypes.c_int, P, ctypes.c_int, P, ctypes.POINTER(ctypes.c_int)]
            g.restype = ctypes.c_int
    return _lib


def ref_available():
    return os.path.exists(_REF) and _arch_ok(_REF)


def _load_ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref/libcp3ref.so is not built on this machine")
        _ref = ctypes.CDLL(_REF)
        for sfx, ct in (("_f64", ctypes.c_double), ("_f32", ctypes.c_float)):
            f = getattr(_ref, "ref_calculate" + sfx)
            P = ctypes.POINTER(ct)
            f.argtypes = [ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P, P,
                          ct, ct, ct, ct, ct, ct, ct, ctypes.c_int, ctypes.c_int, P]
            f.restype = ctypes.c_int
        _ref.ref_last_error.restype = ctypes.c_char_p
    return _ref


def max_threads():
    return int(_load().oracle_max_threads())


def _call(fn, dtype, cosines, energies, radii, rhos, params, height_km, anti, threads, planar):
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    P = ctypes.POINTER(ct)
    c = np.ascontiguousarray(cosines, dtype=dtype)
    e = np.ascontiguousarray(energies, dtype=dtype)
    r = np.ascontiguousarray(radii, dtype=dtype)
    d = np.ascontiguousarray(rhos, dtype=dtype)
    out = np.empty((c.size, e.size, 9), dtype=dtype)
    th12, th13, th23, dcp, dm12, dm23 = params
    rc = fn(c.size, c.ctypes.data_as(P), e.size, e.ctypes.data_as(P), r.size,
            r.ctypes.data_as(P), d.ctypes.data_as(P), th12, th13, th23, dcp, dm12, dm23,
            height_km, 1 if anti else 0, int(threads), out.ctypes.data_as(P))
    if rc != 0:
        raise RuntimeError("oracle error %d" % rc)
    if planar:
        return np.ascontiguousarray(out.transpose(2, 0, 1))
    return out


def calculate(cosines, energies, radii, rhos, params, height_km=22.0, anti=False,
              threads=0, precision="f64", planar=True):
    """Probabilities from the C restatement.

    ``params`` = (theta12, theta13, theta23, dcp, dm12sq, dm23sq).  Returns
    planar ``[9][n_cos][n_en]`` (index in*3+out, like the GPU layout of
    physics.hpp:689-691) or AoS ``[n_cos][n_en][9]`` when ``planar`` is False.
    """
    lib = _load()
    dtype = np.float64 if precision == "f64" else np.float32
    fn = lib.oracle_calculate_f64 if precision == "f64" else lib.oracle_calculate_f32
    return _call(fn, dtype, cosines, energies, radii, rhos, params, height_km, anti, threads,
                 planar)


def ref_calculate(cosines, energies, radii, rhos, params, height_km=22.0, anti=False,
                  threads=0, precision="f64", planar=True):
    """Probabilities from the reference's own CpuPropagator (oracle/_ref)."""
    lib = _load_ref()
    dtype = np.float64 if precision == "f64" else np.float32
    fn = lib.ref_calculate_f64 if precision == "f64" else lib.ref_calculate_f32
    try:
        return _call(fn, dtype, cosines, energies, radii, rhos, params, height_km, anti,
                     threads if threads > 0 else os.cpu_count(), planar)
    except RuntimeError:
        raise RuntimeError(lib.ref_last_error().decode())


def maxlayers(cosines, radii, precision="f64"):
    lib = _load()
    dtype = np.float64 if precision == "f64" else np.float32
    ct = ctypes.c_double if dtype == np.float64 else ctypes.c_float
    P = ctypes.POINTER(ct)
    c = np.ascontiguousarray(cosines, dtype=dtype)
    r = np.ascontiguousarray(radii, dtype=dtype)
    out = np.empty(c.size, dtype=np.int32)
    fn = lib.oracle_maxlayers_f64 if precision == "f64" else lib.oracle_maxlayers_f32
    rc = fn(c.size, c.ctypes.data_as(P), r.size, r.ctypes.data_as(P),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc != 0:
        raise RuntimeError("oracle error %d" % rc)
    return out

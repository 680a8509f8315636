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


def build(ref_dir=None):
    """Compile liboracle.so, and oracle/_ref when ``ref_dir`` (default: the
    REF_DIR environment variable) names the reference's source directory."""
    env = dict(os.environ)
    if ref_dir:
        env["REF_DIR"] = ref_dir
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
        P = ctypes.POINTER(ctypes.c_double)
        d = ctypes.c_double
        _ref.ref_calculate_file_f64.argtypes = [ctypes.c_int, P, ctypes.c_int, P, ctypes.c_char_p, d, d, d, d, d, d,
                                                d, ctypes.c_int, ctypes.c_int, P]
        _ref.ref_calculate_file_f64.restype = ctypes.c_int
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


def ref_calculate_file(cosines, energies, path, params, height_km=22.0, anti=False, threads=0, planar=True):
    """Probabilities from the reference's own CpuPropagator<double> with the
    body read by its setDensityFromFile from ``path`` (oracle/_ref)."""
    lib = _load_ref()
    P = ctypes.POINTER(ctypes.c_double)
    c = np.ascontiguousarray(cosines, dtype=np.float64)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    out = np.empty((c.size, e.size, 9), dtype=np.float64)
    th12, th13, th23, dcp, dm12, dm23 = params
    rc = lib.ref_calculate_file_f64(c.size, c.ctypes.data_as(P), e.size, e.ctypes.data_as(P),
                                    os.fsencode(path), th12, th13, th23, dcp, dm12, dm23, height_km,
                                    1 if anti else 0, threads if threads > 0 else os.cpu_count(),
                                    out.ctypes.data_as(P))
    if rc != 0:
        raise RuntimeError(lib.ref_last_error().decode())
    return np.ascontiguousarray(out.transpose(2, 0, 1)) if planar else out


_REF_GPU_CUBIN = os.path.join(_HERE, "_ref", "ref_kernels.cubin")
_REF_GPU_DRIVER = os.path.join(_HERE, "_ref", "ref_gpu_driver")


def _ref_gpu_inputs(precision, anti):
    return os.path.join(_HERE, "_ref", "refgpu_%s_%s.bin" % (precision, "nubar" if anti else "nu"))


def ref_gpu_status():
    """None when the reference's CUDA kernel can be launched here (its cubin,
    the inputs of the benchmark grid and the loader are present), else the
    reason it cannot."""
    if not os.path.exists(_REF_GPU_CUBIN):
        return "oracle/_ref/ref_kernels.cubin absent (built only where the reference sources are)"
    for p in ("f64", "f32"):
        for anti in (False, True):
            if not os.path.exists(_ref_gpu_inputs(p, anti)):
                return "oracle/_ref inputs of the reference kernel absent"
    if not os.path.exists(_REF_GPU_DRIVER):
        return "oracle/_ref/ref_gpu_driver not built"
    return None


def ref_gpu_run(precision="f64", anti=False, reps=5, stride=32):
    """Launch the reference's calculateKernel<double|float> on the 4096 x 4096
    benchmark grid through oracle/_ref/ref_gpu_driver; returns the driver's
    JSON record (per-launch milliseconds, median, registers, local bytes) and
    every ``stride``-th cosine and energy of its nine planes [9][nc][ne]."""
    import json
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "subset.bin")
        r = subprocess.run([_REF_GPU_DRIVER, _REF_GPU_CUBIN, _ref_gpu_inputs(precision, anti), str(reps), out,
                            str(stride)], capture_output=True, text=True, timeout=600)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        rec = json.loads(lines[-1]) if lines else {"error": (r.stderr or "no output").strip()[-300:]}
        if r.returncode != 0 or "error" in rec:
            raise RuntimeError("reference kernel: %s" % rec.get("error", "exit %d" % r.returncode))
        sub = np.fromfile(out, dtype=np.float64).reshape(rec["subset"])
    return rec, sub


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

"""ctypes binding of libcudaprob3_gb300.so (the C ABI of include/cudaprob3_gb300.h).

The library is built in-tree by cudaprob3_gb300.build.  Loading fails loudly
when it is missing: there is no CPU implementation behind this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# CUDAPROB3_GB300_LIBRARY selects another build of the same library, e.g. the
# bounds-checked libcudaprob3_gb300_check.so
LIB_PATH = os.environ.get("CUDAPROB3_GB300_LIBRARY") or os.path.join(HERE, "libcudaprob3_gb300.so")
CHECK_LIB_PATH = os.path.join(HERE, "libcudaprob3_gb300_check.so")

# status codes (include/cudaprob3_gb300.h)
OK = 0
ERR_ARGUMENT = -1
ERR_STATE = -2
ERR_CUDA = -3
ERR_NO_DEVICE = -4
ERR_FILE = -5
ERR_LIMIT = -6
ERR_CHECK = -7

PRECISION_FP64 = 0
PRECISION_MIXED = 1

# (name, restype, argtypes) of every exported entry point
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_SZ = ctypes.c_size_t
SIGNATURES = [
    ("cp3_abi_version", _I, []),
    ("cp3_bounds_checked", _I, []),
    ("cp3_last_error", ctypes.c_char_p, []),
    ("cp3_device_count", _I, []),
    ("cp3_create", _I, [ctypes.POINTER(_P), _I, _I, _I, _I]),
    ("cp3_destroy", _I, [_P]),
    ("cp3_set_energy_list", _I, [_P, _DP, _I]),
    ("cp3_set_cosine_list", _I, [_P, _DP, _I]),
    ("cp3_set_mns_matrix", _I, [_P, _D, _D, _D, _D]),
    ("cp3_set_neutrino_masses", _I, [_P, _D, _D]),
    ("cp3_set_density", _I, [_P, _DP, _DP, _DP, _I]),
    ("cp3_set_density_from_file", _I, [_P, ctypes.c_char_p]),
    ("cp3_set_production_height", _I, [_P, _D]),
    ("cp3_set_production_heights", _I, [_P, _DP, _DP, _I]),
    ("cp3_calculate_probabilities", _I, [_P, _I]),
    ("cp3_calculate_probabilities_async", _I, [_P, _I]),
    ("cp3_wait_for_completion", _I, [_P]),
    ("cp3_get_probability", _I, [_P, _I, _I, _I, _DP]),
    ("cp3_result_device_ptr", _I, [_P, ctypes.POINTER(_P)]),
    ("cp3_result_bytes", _I, [_P, ctypes.POINTER(_SZ)]),
    ("cp3_copy_results_to_host", _I, [_P, _P, _SZ]),
    ("cp3_set_result_buffer", _I, [_P, _P, _SZ]),
    ("cp3_set_host_result_buffer", _I, [_P, _P, _SZ]),
    ("cp3_set_host_completion", _I, [_P, _I]),
    ("cp3_set_rate_flux", _I, [_P, _P, _I, _I]),
    ("cp3_set_rate_bins", _I, [_P, _IP, _IP, _I, _I]),
    ("cp3_calculate_rates", _I, [_P, _I]),
    ("cp3_calculate_rates_async", _I, [_P, _I]),
    ("cp3_rates_device_ptr", _I, [_P, ctypes.POINTER(_P)]),
    ("cp3_get_rates", _I, [_P, _DP, _SZ]),
    ("cp3_set_stream", _I, [_P, _P]),
    ("cp3_last_launch_count", _I, [_P, _IP]),
    ("cp3_get_maxlayers", _I, [_P, _IP, _I]),
    ("cp3_set_launch_shape", _I, [_P, _I, _I, _I]),
    ("cp3_get_launch_shape", _I, [_P, _IP, _IP, _IP]),
    ("cp3_autotune", _I, [_P, _I, _I, _IP, _IP, _IP, ctypes.POINTER(ctypes.c_float)]),
    ("cp3_set_kernel_timing", _I, [_P, _I]),
    ("cp3_last_kernel_ms", _I, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    ("cp3_batch_create", _I, [ctypes.POINTER(_P), _I, _I, _I, _IP, _IP]),
    ("cp3_batch_destroy", _I, [_P]),
    ("cp3_batch_set_grids", _I, [_P, _DP, _DP]),
    ("cp3_batch_set_parameters", _I, [_P, _DP]),
    ("cp3_batch_set_density", _I, [_P, _DP, _DP, _DP, _I, _DP]),
    ("cp3_batch_set_production_height", _I, [_P, _D]),
    ("cp3_batch_set_stream", _I, [_P, _P]),
    ("cp3_batch_set_launch_shape", _I, [_P, _I, _I, _I]),
    ("cp3_batch_get_launch_shape", _I, [_P, _IP, _IP, _IP, _IP]),
    ("cp3_batch_autotune", _I, [_P, _I, _I, _IP, _IP, _IP, ctypes.POINTER(ctypes.c_float)]),
    ("cp3_batch_calculate", _I, [_P, _I]),
    ("cp3_batch_calculate_async", _I, [_P, _I]),
    ("cp3_batch_wait", _I, [_P]),
    ("cp3_batch_calculate_sequential", _I, [_P, _I]),
    ("cp3_batch_last_ms", _I, [_P, ctypes.POINTER(ctypes.c_float)]),
    ("cp3_batch_launch_count", _I, [_P, _I, _IP]),
    ("cp3_batch_result_offsets", _I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("cp3_batch_result_device_ptr", _I, [_P, ctypes.POINTER(_P)]),
    ("cp3_batch_copy_results_to_host", _I, [_P, _P, _SZ]),
    ("cp3_batch_get_maxlayers", _I, [_P, _IP, ctypes.c_longlong]),
    ("cp3_loglik_create", _I, [ctypes.POINTER(_P), _I, _I, _I, _I]),
    ("cp3_loglik_destroy", _I, [_P]),
    ("cp3_loglik_set_bins", _I, [_P, _DP, _DP]),
    ("cp3_loglik_set_body", _I, [_P, _DP, _DP, _I]),
    ("cp3_loglik_set_production_height", _I, [_P, _D]),
    ("cp3_loglik_set_flux", _I, [_P, _DP, _DP, _D]),
    ("cp3_loglik_set_observed", _I, [_P, _DP]),
    ("cp3_loglik_evaluate", _I, [_P, _I, _DP, _DP, _DP, _DP]),
    ("cp3_loglik_set_kernel_timing", _I, [_P, _I]),
    ("cp3_loglik_last_kernel_ms", _I, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float)]),
    ("cp3_loglik_io_bytes", _I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    ("cp3_propagate_noalloc", _I, [_I, _I, _P, _I, _P, _I, _DP, _DP, _DP, _I, _D, _D, _D, _D, _D, _D, _D, _P,
                                   _P]),
]

_lib = None


class CP3Error(RuntimeError):
    """Error raised for a non-zero status of the C ABI (the reference throws
    std::runtime_error with the same message)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def load():
    """Load the shared library; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("%s is not built: run `python -m cudaprob3_gb300.build`" % os.path.basename(LIB_PATH))
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc):
    if rc != OK:
        raise CP3Error(rc, load().cp3_last_error().decode())
    return rc

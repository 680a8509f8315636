"""The C ABI library without a GPU: it loads, exports every declared symbol,
and reports errors through status codes."""
import ctypes
import os
import re

import pytest

import cudaprob3_gb300 as cp
from cudaprob3_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "cudaprob3_gb300.h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(cp3_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_library_loads():
    lib = cp.load_library()
    assert lib.cp3_abi_version() == 1


@pytest.mark.parametrize("name", declared_symbols())
def test_symbol_exported(name):
    lib = ctypes.CDLL(_lib.LIB_PATH)
    assert hasattr(lib, name)


def test_binding_covers_header():
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_null_handle_errors():
    lib = cp.load_library()
    assert lib.cp3_set_production_height(None, 1.0) == _lib.ERR_ARGUMENT
    assert b"null" in lib.cp3_last_error()
    assert lib.cp3_destroy(None) == 0


def test_create_without_device():
    if cp.device_count() > 0:
        pytest.skip("a device is visible")
    with pytest.raises(cp.CP3Error) as e:
        cp.CudaPropagatorSingle(0, 8, 8)
    assert e.value.code == _lib.ERR_NO_DEVICE
    assert "No GPU found" in str(e.value)


def test_bad_precision_rejected():
    with pytest.raises(ValueError):
        cp.CudaPropagatorSingle(0, 8, 8, precision="half")


def product_files():
    """Every source file of the shipped product: package, kernels, headers."""
    for top in ("cudaprob3_gb300", "include"):
        for d, _, files in os.walk(os.path.join(ROOT, top)):
            if "__pycache__" in d:
                continue
            for f in files:
                if f.endswith((".py", ".cu", ".cuh", ".h", ".hpp", ".cpp")):
                    yield os.path.join(d, f)


def test_product_never_touches_the_oracle():
    # the oracle serves the tests and the CPU legs of bench.py only
    hits = [p for p in product_files() if re.search(r"\boracle\b", open(p).read())]
    assert not hits, hits


def test_missing_library_fails_loudly(monkeypatch):
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", os.path.join(ROOT, "no_such_dir", "libcudaprob3_gb300.so"))
    with pytest.raises(ImportError, match="not built"):
        _lib.load()


def test_binding_arity_matches_header():
    """Every ctypes signature has as many arguments as the C declaration."""
    text = "".join(open(h).read() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    decls = re.findall(r"(?:int|const char\s*\*)\s+(cp3_\w+)\s*\(([^)]*)\)\s*;", text, re.S)
    assert decls
    arity = {n: len(args) for n, _, args in _lib.SIGNATURES}
    for name, params in decls:
        p = params.strip()
        n = 0 if p in ("", "void") else p.count(",") + 1
        assert arity[name] == n, (name, n, arity[name])

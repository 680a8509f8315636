"""Build recipe of the CUDA library (sm_103a) and its C++ drop-in example.

    python -m cudaprob3_gb300.build          # libcudaprob3_gb300.so in-tree

The library is compiled with nvcc directly (no torch extension machinery):
one -gencode for sm_103a, one process per translation unit, then a link step.
The same call builds the bounds-checked debug library
libcudaprob3_gb300_check.so (the same sources with -DCP3_CHECK: every kernel
index compared with its buffer's extent, failures reported as CP3_ERR_CHECK;
select it with CUDAPROB3_GB300_LIBRARY=<path>) and the benchmark's pipe
probes (bench_pipes.cu beside bench.py) into libbench_pipes.so, a library of
their own.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcudaprob3_gb300.so")
# the bounds-checked debug build of the same sources (-DCP3_CHECK)
BUILD_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(HERE, "libcudaprob3_gb300_check.so")
SOURCES = ["cp3_abi.cu", "cp3_kernels.cu", "cp3_batch.cu", "cp3_loglik.cu", "cp3_noalloc.cu"]
# the benchmark's pipe-throughput probes: a library of their own, not part of
# the propagator's library or public header
BENCH_PIPES_SRC = os.path.join(ROOT, "bench_pipes.cu")
BENCH_PIPES_LIB = os.path.join(ROOT, "libbench_pipes.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-fopenmp", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "cudaprob3_gb300.h"))
    return hs


def _loads_here(path):
    import ctypes
    try:
        ctypes.CDLL(path)
        return True
    except OSError:
        return False


def build(verbose=False, force=False, check=True):
    """Compile every translation unit for sm_103a and link the shared library
    (and, with check, the bounds-checked library), all nvcc processes in
    parallel."""
    heads = _headers()
    jobs = []
    links = []
    for build_dir, lib, extra in ((BUILD, LIB, []), (BUILD_CHECK, LIB_CHECK, ["-DCP3_CHECK"]))[:2 if check else 1]:
        os.makedirs(build_dir, exist_ok=True)
        objs = []
        fresh = True
        for src in SOURCES:
            s = os.path.join(CSRC, src)
            o = os.path.join(build_dir, src.replace(".cu", ".o"))
            objs.append(o)
            if force or not _newer(o, [s] + heads):
                jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o])
                fresh = False
        if force or not fresh or not _newer(lib, objs) or not _loads_here(lib):
            links.append([nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", lib] + objs)
    if force or not _newer(BENCH_PIPES_LIB, [BENCH_PIPES_SRC]) or not _loads_here(BENCH_PIPES_LIB):
        jobs.append([nvcc()] + ARCH + ["-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", BENCH_PIPES_SRC,
                                       "-o", BENCH_PIPES_LIB])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr
    with ThreadPoolExecutor(max_workers=max(1, len(jobs), len(links))) as ex:
        list(ex.map(run, jobs))
        list(ex.map(run, links))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

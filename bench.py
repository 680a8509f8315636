"""Throughput benchmark of the GB300 Barger propagator.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): the 4096-cosine x 4096-energy grid (cosines uniform in
[-1, 0], energies log-spaced over 0.1-1000 GeV), 11-shell PREM body with
electron fractions 0.468 (core) / 0.497 (mantle), nominal oscillation point,
production height 22 km, computed for neutrinos AND antineutrinos (two
calculateProbabilities calls, 2 x 16.8M pairs).  Metric: (cos, E) pairs/s.

Our arm runs the mixed-precision kernel (double-float eigen-solve, Q1.30 fixed-point
chain, float results) and reports beside it the plain FP64 kernel on the same
workload, the precision of mixed against FP64 (every pair) and against the
oracle (strided subset), the roofline of the dominant kernel and the CPU
baseline.  The reference arm times the reference's CPU path (the oracle's C
restatement of CpuPropagator<double>, all host threads) on a bounded sample of
the same workload.

N > 1 (torchrun): every rank runs the same workload on its own GPU (replicas,
weak scaling; the path has no exchange step); value = all ranks' pairs / the
slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NC = NE = 4096
E_MIN, E_MAX = 0.1, 1000.0
WORKLOAD = ("4096 cos x 4096 E (cos in [-1,0], 0.1-1000 GeV log), 11-shell PREM "
            "(Ye 0.468 core / 0.497 mantle), nominal parameters, h=22 km, nu + nubar per step")
METRIC = "(cos,E) pairs/s on 1 GB300: mixed-precision vs plain FP64 at max|dP|<=1e-6"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="target CPU time of the baseline sample")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--precision-sets", type=int, default=64,
                    help="parameter sets of the 8192 x 8192 precision table in the default line (0: skip)")
    ap.add_argument("--workload", choices=["grid4096", "batch", "precision", "gradient", "rates", "heights"],
                    default="grid4096",
                    help="grid4096: the headline line; batch: 1024 parameter sets with uneven grids in one "
                         "graph launch; precision: 64 parameter sets on the 8192 x 8192 grid")
    ap.add_argument("--sets", type=int, default=0, help="number of parameter sets (batch/precision)")
    # one small case for profilers (ncu): no timing contract, no JSON line
    ap.add_argument("--profile-case", choices=["planes", "rates", "heights", "gradient", "bands"], default=None,
                    help="run one square grid (or the gradient evaluation, or fixed-layer-count bands) for a "
                         "profiler instead of a benchmark")
    ap.add_argument("--bands", type=int, nargs="*", default=[2, 3, 4, 7, 11],
                    help="profile case bands: crossed-shell counts M, one launch each")
    ap.add_argument("--n", type=int, default=2048, help="profile case: cosines = energies")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed", help="profile case: arithmetic")
    ap.add_argument("--repeat", type=int, default=1, help="profile case: calculations")
    ap.add_argument("--anti", action="store_true", help="profile case: antineutrinos")
    return ap.parse_args()


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def grid():
    from cudaprob3_gb300 import grids as G
    return G.linspace(-1.0, 0.0, NC), G.logspace(E_MIN, E_MAX, NE), G.PREM_12, G.NOMINAL


# ------------------------------------------------------------- work units --
def products_per_pair(M):
    """32x32 -> 64 integer products (mul.wide.s32) of one pair in the mixed
    kernel's algorithm (flavour_block in cp3_chain.cuh), every complex product
    counted as four real ones: 52 per inner chain step T_l D_l on two columns,
    36 to rebuild the third column, and the fixed cost of D_0 Gamma', T_0 (.),
    G = Y^T D_M Y, G X', Lambda' X and the four exact |S|^2 of the 2x2 flavour
    block.  The kernel forms complex products with Gauss's three products, so
    it executes fewer (48 per inner step); the roofline counts this fixed
    algorithmic work."""
    M = np.asarray(M, dtype=np.int64)
    return np.where(M >= 2, 52 * M + 198, np.where(M == 1, 260, 68))


def reference_flops_per_pair(M):
    """Per-pair algorithmic work of the reference formulation,
    F = (M+1)*(3 + 216 + 3) + n_mm*216 + 27 with n_mm = 2M (M >= 1) or 1."""
    M = np.asarray(M, dtype=np.int64)
    nmm = np.where(M >= 1, 2 * M, 1)
    return (M + 1) * 222 + nmm * 216 + 27


def ll_pair_products_per_pair(M):
    """Real multiply-adds of one (cosine, energy) bin in ll_pair_kernel
    (cp3_loglik.cu): the forward chain (D_0 Gamma', T_0, the inner steps
    U = D_l Y, Y = T_l U, G = Y^T D_M Y, G X', the 2x2 block, |B|^2) plus the
    adjoint (the seeds, the adjoints of X, Lambda', G, x, T_0, Gamma', D_0,
    Y and D_M, and per crossed shell the un-multiplied chain and its
    adjoint), every complex product counted as four real ones and every real
    times complex as two; phase evaluations and warp sums are not counted.
    For M >= 2 crossed shells: 400 + 90 (M - 2) forward and 874 + 278 (M - 2)
    backward."""
    M = np.asarray(M, dtype=np.int64)
    return np.where(M >= 2, 1274 + 368 * (M - 2), np.where(M == 1, 1086, 178))


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one
# propagate_kernel<mixed> launch per pair, from one ncu capture of the
# 4096 x 4096 launch, and the SHA-256 of the device sources the kernel was
# compiled from at that capture.  When the sources differ the figure no longer
# describes the kernel, and the roofline's traffic is reported as null.
TRAFFIC_BYTES_PER_PAIR = 545_107_456 / (4096 * 4096)
TRAFFIC_SOURCES_SHA = "e2a73aab19dcd86ea68ae1db85074d79d8ee7ea7395b4daab9036948df4e4a7b"
TRAFFIC_SOURCES = ("cp3_arith.cuh", "cp3_chain.cuh", "cp3_check.cuh", "cp3_df.cuh", "cp3_internal.h",
                   "cp3_kernels.cu", "cp3_physics.cuh", "cp3_tile.cuh")


def traffic_sources_sha():
    """SHA-256 over the sources the propagate kernel is compiled from (its
    body, its launch bounds and the helpers it inlines)."""
    import hashlib
    h = hashlib.sha256()
    for name in TRAFFIC_SOURCES:
        with open(os.path.join(ROOT, "cudaprob3_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


# ------------------------------------------------------------- pipe peaks --
def pipe_peak(pipe, device):
    """(operations/s, SM MHz during the probe, SM count) of one pipe -- 0
    mul.wide.s32 integer products, 1 FP32 FMA, 2 FP64 FMA -- from the
    benchmark's own probe library (bench_pipes.cu, built by build())."""
    import ctypes
    path = os.path.join(ROOT, "libbench_pipes.so")
    lib = ctypes.CDLL(path)
    lib.bench_pipe_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    lib.bench_pipe_peak.restype = ctypes.c_int
    ops, mhz, sms = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    rc = lib.bench_pipe_peak(int(device), int(pipe), ctypes.byref(ops), ctypes.byref(mhz), ctypes.byref(sms))
    if rc != 0:
        raise RuntimeError("pipe probe failed with CUDA error %d" % rc)
    return ops.value, mhz.value, sms.value


PIPE_IMAD_WIDE, PIPE_FFMA, PIPE_DFMA = 0, 1, 2


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        power = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(power) if power else None}


# -------------------------------------------------------------- CPU legs --
def cpu_sample(target_s, threads=0):
    """Time the oracle (CpuPropagator<double> restated) on whole cosine rows of
    the workload, nu and nubar alternately, until about `target_s` seconds.
    Returns (pairs/s, threads, description)."""
    import oracle
    cos, en, B, nom = grid()
    threads = threads or os.cpu_count() or 1
    rows = 0
    pairs = 0
    t_total = 0.0
    k = 0
    while t_total < target_s and k < NC // 16:
        c = cos[(np.arange(16) * (NC // 16) + k) % NC]
        t0 = time.perf_counter()
        oracle.calculate(c, en, B.radii, B.rho_eff(), nom, 22.0, bool(k % 2), threads=threads)
        t_total += time.perf_counter() - t0
        pairs += c.size * en.size
        rows += c.size
        k += 1
    desc = "%d cosine rows x %d energies (strided over the grid, nu/nubar alternating), %.1f s" % (
        rows, NE, t_total)
    return pairs / t_total, threads, desc


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    cos, en, B, nom = grid()
    threads = os.cpu_count() or 1
    rows_per_step = 16
    times = []
    for s in range(args.warmup + args.steps):
        c = cos[(np.arange(rows_per_step) * (NC // rows_per_step) + s) % NC]
        t0 = time.perf_counter()
        for anti in (False, True):
            oracle.calculate(c, en, B.radii, B.rho_eff(), nom, 22.0, anti, threads=threads)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    pairs = 2 * rows_per_step * NE * len(times)
    value = pairs / sum(times)
    sample = ("per step: %d cosine rows x %d energies, nu and nubar (%d pairs of the 2x16.8M)"
              % (rows_per_step, NE, 2 * rows_per_step * NE))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


# ------------------------------------------------- the reference's kernel --
def reference_gpu_leg(value, fp64_value):
    """The reference's own CUDA kernel, calculateKernel<double> and <float>
    (physics.hpp:705-721), recompiled for sm_103a, launched as
    CudaPropagatorSingle launches it (64-thread blocks) on the same 4096 x 4096
    grid, body and parameters as the headline, nu and nubar, with the constants
    and device arrays its own host code prepared (oracle/ref_gpu_kernel.cu,
    ref_gpu_inputs.cpp, ref_gpu_driver.cpp): per type the median of 5 timed
    launches (CUDA events) after one warm-up; outputs (1.2 GB / 0.6 GB per
    launch) exceed L2.  Errors against the oracle on every 32nd cosine and
    energy; the float kernel gets the grid and body rounded to float."""
    import oracle
    status = oracle.ref_gpu_status()
    if status:
        return {"unavailable": status}
    cos, en, B, nom = grid()
    idx = np.arange(0, NC, 32)
    want = {anti: oracle.calculate(cos[idx], en[idx], B.radii, B.rho_eff(), nom, 22.0, anti) for anti in (False, True)}
    out = {"workload": WORKLOAD, "launch": "calculateKernel<T>, 64-thread blocks, ceil(nE/64)*nC blocks, one launch "
                                          "per neutrino type (cudapropagator.cuh:191-220)",
           "timing": "median of 5 launches per type after a warm-up, CUDA events; step = nu + nubar"}
    try:
        for prec, name in (("f64", "double"), ("f32", "float")):
            ms = 0.0
            err = 0.0
            mean = 0.0
            rec = None
            for anti in (False, True):
                rec, sub = oracle.ref_gpu_run(prec, anti, reps=5, stride=32)
                ms += rec["median_ms"]
                d = np.abs(sub - want[anti])
                err = max(err, float(d.max()))
                mean += float(d.mean()) / 2
            out[name] = {"pairs_per_s": 2 * NC * NE / (ms * 1e-3), "ms_per_step": ms,
                         "max_abs_dp_vs_oracle_subset": err, "mean_abs_dp_vs_oracle_subset": mean,
                         "registers": rec["registers"], "local_bytes_per_thread": rec["local_bytes"]}
    except (RuntimeError, OSError, ValueError, KeyError) as exc:
        return {"unavailable": "the reference kernel did not run: %s" % str(exc)[:300]}
    out["mixed_speedup_vs_reference_double"] = value / out["double"]["pairs_per_s"]
    out["mixed_speedup_vs_reference_float"] = value / out["float"]["pairs_per_s"]
    if fp64_value:
        out["fp64_speedup_vs_reference_double"] = fp64_value / out["double"]["pairs_per_s"]
    return out


# ------------------------------------------------------------------- ours --
def make_prop(cp, precision, cos, en, B, nom, device):
    p = cp.CudaPropagatorSingle(device, len(cos), len(en), precision=precision)
    p.setEnergyList(en)
    p.setCosineList(cos)
    p.setMNSMatrix(*nom[:4])
    p.setNeutrinoMasses(*nom[4:])
    p.setDensity(B.radii, B.rhos, B.ye)
    p.setProductionHeight(22.0)
    return p


def small_case(cp, dev):
    """The reference's CPU-runnable case (256 cos x 256 E over 0.5-100 GeV,
    4-shell body, neutrinos): GPU mixed and FP64 (one calculation, CUDA events
    on the handle's stream, best of 20) against the CPU port with all host
    threads (min of 3 after a warm-up) on the whole grid."""
    import torch

    import oracle
    from cudaprob3_gb300 import grids as G
    n = 256
    cos = G.linspace(-1.0, 0.0, n)
    en = G.logspace(0.5, 100.0, n)
    B = G.PREM_4
    out = {"workload": "256 cos x 256 E (0.5-100 GeV), 4-shell body, nominal parameters, nu"}
    for precision in ("mixed", "fp64"):
        p = make_prop(cp, precision, cos, en, B, G.NOMINAL, dev)
        s = torch.cuda.Stream(device=dev)
        p.set_stream(s.cuda_stream)
        best = 1e30
        for _ in range(20):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(s)
            p.calculateProbabilitiesAsync(cp.Neutrino)
            b.record(s)
            b.synchronize()
            best = min(best, a.elapsed_time(b))
        out["gpu_%s_pairs_per_s" % precision] = n * n / (best * 1e-3)
        p.close()
    threads = os.cpu_count() or 1
    oracle.calculate(cos, en, B.radii, B.rho_eff(), G.NOMINAL, 22.0, False, threads=threads)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        oracle.calculate(cos, en, B.radii, B.rho_eff(), G.NOMINAL, 22.0, False, threads=threads)
        ts.append(time.perf_counter() - t0)
    out["cpu_port_pairs_per_s"] = n * n / min(ts)
    out["cpu_cores"] = threads
    out["note"] = "a 65,536-pair grid is launch-bound on the GPU"
    return out


def run_ours(args, world, rank, local):
    import torch

    import cudaprob3_gb300 as cp

    dev = local
    torch.cuda.set_device(dev)
    cos, en, B, nom = grid()
    stream = torch.cuda.Stream(device=dev)
    stream2 = torch.cuda.Stream(device=dev)  # the antineutrino handle: its prep overlaps the neutrino kernel
    streams = (stream, stream2)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def build(precision):
        props = []
        bufs = []
        dt = torch.float32 if precision == "mixed" else torch.float64
        for anti in (False, True):
            p = make_prop(cp, precision, cos, en, B, nom, dev)
            buf = torch.empty((9, NC, NE), dtype=dt, device=dev)
            p.set_result_buffer(buf.data_ptr(), buf.numel() * buf.element_size())
            p.set_stream(streams[int(anti)].cuda_stream)
            props.append((p, cp.Antineutrino if anti else cp.Neutrino))
            bufs.append(buf)
        return props, bufs

    def timed_steps(props, steps, warmup, kernel_times=None):
        # one step: both types, each handle on its own stream (fork and join
        # by events inside the timed region).  With kernel_times, both handles
        # run on one stream instead, so that each kernel's events time it alone.
        serial = kernel_times is not None
        if serial:
            for p, _ in props:
                p.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                for p, t in props:
                    p.calculateProbabilitiesAsync(t)
            torch.cuda.synchronize()
            evs = []
            barrier(world)
            torch.cuda.synchronize()
            for _ in range(steps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                j = torch.cuda.Event()
                a.record(stream)
                stream2.wait_event(a)
                for p, t in props:
                    p.calculateProbabilitiesAsync(t)
                j.record(stream2)
                stream.wait_event(j)
                b.record(stream)
                evs.append((a, b))
                if kernel_times is not None:
                    for p, _ in props:
                        kernel_times.append(p.last_kernel_ms())
            torch.cuda.synchronize()
            barrier(world)
        if serial:
            for i, (p, _) in enumerate(props):
                p.set_stream(streams[i].cuda_stream)
        return [a.elapsed_time(b) for a, b in evs]

    # ---- mixed: the headline
    props, bufs = build("mixed")
    maxl = props[0][0].maxlayers()
    sampler = ClockSampler(dev)
    sampler.start()
    times = timed_steps(props, args.steps, args.warmup)
    clocks = sampler.stop()
    # each kernel alone (serialised pass) for the roofline
    for p, _ in props:
        p.set_kernel_timing(True)
    kt = []
    timed_steps(props, max(5, min(args.steps, 50)), 1, kt)
    for p, _ in props:
        p.set_kernel_timing(False)
    ms_step = allmax(world, sum(times) / len(times))
    pairs_step = 2 * NC * NE
    value = world * pairs_step / (ms_step * 1e-3)
    launches = sum(p.last_launch_count() for p, _ in props) * args.steps

    prop_ms = float(np.mean([k[1] for k in kt]))
    prep_ms = float(np.mean([k[0] for k in kt]))
    prods = float(products_per_pair(maxl).sum()) * NE
    peak_prod, prod_mhz, n_sm = pipe_peak(PIPE_IMAD_WIDE, dev)
    peak_ffma, _, _ = pipe_peak(PIPE_FFMA, dev)
    peak_dfma, dfma_mhz, _ = pipe_peak(PIPE_DFMA, dev)
    out_bytes = 9 * NC * NE * 4
    ref_f = float(reference_flops_per_pair(maxl).sum()) * NE
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak, hbm_src = float(mp["hbm_gbs"]), "MEASURED_PEAKS.json (measured)"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback 6.8 TB/s"
    # DRAM bytes of one launch: the captured per-pair figure times this
    # launch's pairs, while the kernel's sources are those of the capture
    sources_sha = traffic_sources_sha()
    traffic_current = sources_sha == TRAFFIC_SOURCES_SHA
    traffic = TRAFFIC_BYTES_PER_PAIR * NC * NE if traffic_current else None
    roofline = {
        "bound": "fma-pipe (mul.wide.s32 integer products on the FMA-heavy pipe)",
        "achieved": prods / (prop_ms * 1e-3) / 1e12, "peak": peak_prod / 1e12, "unit": "Tops/s",
        "frac": (prods / (prop_ms * 1e-3)) / peak_prod, "traffic": traffic,
        "kernel": "propagate_kernel<mixed>", "kernel_ms": prop_ms, "prep_kernel_ms": prep_ms,
        "work_per_launch": prods,
        "work_unit": "32x32->64 integer products, four-product form of every complex product (products_per_pair)",
        "peak_source": "measured live on this GPU (bench_pipes.cu) at %.0f MHz SM clock, %d SMs" % (prod_mhz, n_sm),
        "traffic_source": ("ncu capture of one 4096^2 launch (%.2f B/pair) x pairs of this launch; kernel sources "
                           "unchanged since (sha %s)" % (TRAFFIC_BYTES_PER_PAIR, sources_sha[:12])) if traffic_current
        else "null: the kernel's device sources changed since the last capture (sha %s)" % sources_sha[:12],
        "algorithmic_out_bytes": out_bytes,
        "hbm_output_gbs": out_bytes / (prop_ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm_peak,
        "hbm_frac": out_bytes / (prop_ms * 1e-3) / 1e9 / hbm_peak, "hbm_peak_source": hbm_src,
        "reference_form_tflops": ref_f / (prop_ms * 1e-3) / 1e12,
        "ffma_peak_tflops": 2 * peak_ffma / 1e12, "dfma_peak_tflops": 2 * peak_dfma / 1e12,
    }

    # ---- e2e through the public API with host buffers: inputs uploaded from
    # host arrays every step, results stored by the kernel straight into
    # page-locked host memory (zero-copy over the host link); the
    # copy-after-kernel form (cudaMemcpy of the planes) is timed beside it
    host = [torch.empty((9, NC, NE), dtype=torch.float32, pin_memory=True) for _ in props]
    cos_h = np.ascontiguousarray(cos)
    en_h = np.ascontiguousarray(en)
    e2e_steps = max(3, min(args.steps, 20))

    def e2e_run(mode):
        # mode "memcpy": planes into the handle's device buffer, then one
        # copy to host; "zero_copy": the kernel stores all nine planes into
        # page-locked host memory; "block": it stores the four planes of the
        # 2x2 flavour block there and waitForCompletion derives the other
        # five on the host cores (set_host_completion)
        for (p, _), h in zip(props, host):
            p.set_stream(0)  # each handle on its own stream
            if mode == "memcpy":
                p.set_result_buffer(0, 0)
            else:
                p.set_host_result_buffer(h.data_ptr(), h.numel() * 4)
            p.set_host_completion(mode == "block")
        for (p, t), h in zip(props, host):  # warm-up
            p.calculateProbabilities(t)
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            if mode != "memcpy":
                # both types in flight on their own streams, one wait each:
                # the second's uploads and prep overlap the first's stores,
                # its stores overlap the first's host completion
                for (p, t), h in zip(props, host):
                    p.setEnergyList(en_h)
                    p.setCosineList(cos_h)
                    p.calculateProbabilitiesAsync(t)
                for p, _ in props:
                    p.waitForCompletion()
            else:
                for (p, t), h in zip(props, host):
                    p.setEnergyList(en_h)
                    p.setCosineList(cos_h)
                    p.calculateProbabilities(t)
                    p.copy_results_to(h.data_ptr(), h.numel() * 4)
        torch.cuda.synchronize()
        dt = allmax(world, (time.perf_counter() - t0) / e2e_steps)
        for i, (p, _) in enumerate(props):
            p.set_host_completion(False)
            p.set_stream(streams[i].cuda_stream)
        return dt

    e2e_memcpy_s = e2e_run("memcpy")
    e2e_block_s = e2e_run("block")
    e2e_s = e2e_run("zero_copy")
    # the host planes of the last e2e step against the device planes of the
    # timed steps (same inputs)
    e2e_dp = max(float((h.to(buf.device) - buf).abs().max()) for h, buf in zip(host, bufs))
    plane_bytes = NC * NE * 4
    e2e = {"value": world * pairs_step / e2e_s, "unit": "pairs/s",
           "h2d_bytes_per_step": 2 * 8 * (NC + NE), "d2h_bytes_per_step": 2 * out_bytes,
           "ms_per_step": e2e_s * 1e3,
           "d2h": "the kernel stores the nine planes into page-locked host buffers (set_host_result_buffer); "
                  "host-timed setEnergyList + setCosineList + calculateProbabilitiesAsync per type on the "
                  "handles' own streams, then waitForCompletion",
           "max_abs_dp_host_vs_device_planes": e2e_dp,
           "copy_after_kernel": {"value": world * pairs_step / e2e_memcpy_s, "ms_per_step": e2e_memcpy_s * 1e3,
                                 "d2h_bytes_per_step": 2 * out_bytes},
           "block_with_host_completion": {
               "value": world * pairs_step / e2e_block_s, "ms_per_step": e2e_block_s * 1e3,
               "d2h_bytes_per_step": 2 * 4 * plane_bytes,
               "note": "four planes over the link, five derived on the host cores (set_host_completion): "
                       "host-memory-bound on this box's cores"}}
    for (p, _), buf in zip(props, bufs):
        p.set_result_buffer(buf.data_ptr(), buf.numel() * 4)

    # ---- plain FP64 on the same workload
    fp64 = None
    prec = {}
    if not args.skip_fp64:
        fprops, fbufs = build("fp64")
        fsteps = max(1, min(args.steps, 3))
        ftimes = timed_steps(fprops, fsteps, 1)
        for p, _ in fprops:
            p.set_kernel_timing(True)
        fkt = []
        timed_steps(fprops, fsteps, 0, fkt)
        for p, _ in fprops:
            p.set_kernel_timing(False)
        fms = allmax(world, sum(ftimes) / len(ftimes))
        fprop_ms = float(np.mean([k[1] for k in fkt]))
        # the same chain in FP64: one DFMA per multiply-add of the mixed
        # kernel's count, against the live-measured DFMA peak of this GPU
        fp64 = {"value": world * pairs_step / (fms * 1e-3), "unit": "pairs/s", "ms_per_step": fms,
                "steps": fsteps,
                "roofline": {"bound": "fp64 pipe (DFMA)", "kernel": "propagate_kernel<fp64>",
                             "kernel_ms": fprop_ms, "work_per_launch": prods,
                             "achieved": prods / (fprop_ms * 1e-3) / 1e12, "peak": peak_dfma / 1e12,
                             "unit": "T DFMA/s", "frac": (prods / (fprop_ms * 1e-3)) / peak_dfma,
                             "note": "chain multiply-adds only; the FP64 phases (257-entry table and "
                                     "Taylor series, 15 FP64 instructions each) and the completion "
                                     "come on top",
                             "peak_source": "measured live on this GPU (bench_pipes.cu) at %.0f MHz SM clock"
                                            % dfma_mhz}}
        # precision of this step's mixed results against FP64 (every pair)
        for p, t in props:
            p.calculateProbabilitiesAsync(t)
        torch.cuda.synchronize()
        dmax, dsum = 0.0, 0.0
        for bm, bf in zip(bufs, fbufs):
            d = (bm.double() - bf).abs()
            dmax = max(dmax, float(d.max()))
            dsum += float(d.mean())
        prec = {"max_abs_dp_vs_fp64": dmax, "mean_abs_dp_vs_fp64": dsum / len(bufs)}
        for p, _ in fprops:
            p.close()
        del fbufs
    if rank == 0:
        import oracle
        idx = np.arange(0, NC, 32)
        err = 0.0
        mean = 0.0
        for k, (p, t) in enumerate(props):
            want = oracle.calculate(cos[idx], en[idx], B.radii, B.rho_eff(), nom, 22.0, bool(t))
            got = bufs[k].cpu().numpy()[:, idx][:, :, idx].astype(np.float64)
            err = max(err, float(np.abs(got - want).max()))
            mean += float(np.abs(got - want).mean()) / 2
        prec["max_abs_dp_vs_oracle_subset"] = err
        prec["mean_abs_dp_vs_oracle_subset"] = mean
        prec["oracle_subset"] = "every 32nd cosine x every 32nd energy (128 x 128), nu and nubar"

    # the precision workload (8192 x 8192, parameter sets of seed 0): mixed
    # against FP64 on every pair, both against the oracle on a subset
    configs2 = None
    if args.precision_sets > 0:
        summary, per_set = precision_sets(dev, args.precision_sets)
        configs2 = dict(summary, per_set=per_set)

    reference_gpu = None
    if rank == 0 and world == 1:
        reference_gpu = reference_gpu_leg(value, fp64["value"] if fp64 else None)

    cpu = None
    configs0 = None
    if rank == 0 and world == 1:
        v, thr, desc = cpu_sample(args.cpu_seconds)
        cpu = {"value": v, "unit": "pairs/s", "cores": thr, "kind": "port", "sample": desc}
        configs0 = small_case(cp, dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "i32 Q1.30 chain + f32 phases + double-float eigen-solve (float out)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "precision": "mixed", "pairs_per_step": pairs_step,
                       "l2": "flushed between steps (256 MB write outside the timed events); "
                             "outputs 2 x 604 MB per step exceed L2",
                       "streams": "nu and nubar handles on two streams, forked and joined by events "
                                  "inside the timed region; the roofline's kernel time comes from a "
                                  "separate pass with both on one stream",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks, "fp64": fp64, "precision": prec,
            "speedup_vs_fp64": (value / fp64["value"]) if fp64 else None,
            "configs0": configs0, "configs2_precision": configs2, "reference_gpu": reference_gpu,
        }
        print(json.dumps(line), flush=True)
    for p, _ in props:
        p.close()


# ------------------------------------------------------------ batch sets --
BATCH_SEED = 3


def batch_sets(n):
    """The batched workload: n parameter sets drawn around the nominal point
    (seed 0, as the precision workload), each with its own grid: cosine count
    uniform-integer 64..1024 over [-1, 0], energy count uniform-integer
    64..2048 log-spaced over 0.5-100 GeV, densities scaled by U(0.97, 1.03)
    (grid sizes and scales from seed 3)."""
    from cudaprob3_gb300 import grids as G
    rng = np.random.default_rng(BATCH_SEED)
    nc = rng.integers(64, 1025, size=n)
    ne = rng.integers(64, 2049, size=n)
    scale = rng.uniform(0.97, 1.03, size=n)
    params = G.draw_parameter_sets(n, seed=0)
    cos = [G.linspace(-1.0, 0.0, int(c)) for c in nc]
    en = [G.logspace(0.5, 100.0, int(e)) for e in ne]
    return nc, ne, params, scale, cos, en


def run_batch(args, world, rank, local):
    import torch

    from cudaprob3_gb300 import grids as G
    from cudaprob3_gb300.batch import BatchPropagator
    import oracle

    torch.cuda.set_device(local)
    n = args.sets or 1024
    nc, ne, params, scale, cos, en = batch_sets(n)
    B = G.PREM_12
    b = BatchPropagator(local, nc, ne, precision="mixed")
    b.set_grids(cos, en)
    b.set_parameters(params)
    b.set_density(B.radii, B.rhos, B.ye, scale)
    b.set_production_height(22.0)
    t0 = time.perf_counter()
    shape, tune_ms = b.autotune(0, reps=1)
    tune_s = time.perf_counter() - t0
    pairs = b.total_pairs
    for _ in range(args.warmup):
        b.calculate(0)
    barrier(world)
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    for k in range(args.steps):
        b.calculate(k % 2)
        times.append(b.last_ms())
    clocks = sampler.stop()
    ms = allmax(world, float(np.mean(times)))
    kernels_per_step = b.launch_count(0)
    seq = []
    for k in range(max(1, min(args.steps, 5))):
        b.calculate_sequential(k % 2)
        seq.append(b.last_ms())
    seq_ms = allmax(world, float(np.mean(seq)))
    # parity of a few sets against the oracle (strided subsets)
    b.calculate(0)
    flat = b.results()
    err = 0.0
    errs = []
    for s_ in range(0, n, max(1, n // 8)):
        got = b.set_result(flat, s_)
        ic = np.arange(0, nc[s_], 16)
        ie = np.arange(0, ne[s_], 16)
        want = oracle.calculate(cos[s_][ic], en[s_][ie], B.radii, B.rho_eff() * scale[s_], tuple(params[s_]),
                                22.0, False)
        d = np.abs(got[:, ic][:, :, ie].astype(np.float64) - want)
        err = max(err, float(d.max()))
        errs.append(float(d.mean()))
    te, groups, cchunk, blocks = b.launch_shape()
    # roofline: the four-product count of every pair of every set (its own
    # grid and layer counts) over the whole graph's time -- the persistent
    # propagate kernel shares that time with the co-running FP64 prep, so the
    # fraction is a lower bound for the propagate kernel alone
    ml = b.maxlayers()
    ne_per_cos = np.repeat(np.asarray(ne, dtype=np.float64), np.asarray(nc, dtype=np.int64))
    prods = float((products_per_pair(ml) * ne_per_cos).sum())
    peak_prod, prod_mhz, n_sm = pipe_peak(PIPE_IMAD_WIDE, local)
    roofline = {"bound": "fma-pipe (mul.wide.s32 integer products on the FMA-heavy pipe)",
                "kernel": "batch_propagate_kernel<mixed> (persistent) with its graph",
                "work_per_launch": prods,
                "work_unit": "32x32->64 integer products, four-product form (products_per_pair) summed over every "
                             "set's pairs",
                "achieved": prods / (ms * 1e-3) / 1e12, "peak": peak_prod / 1e12, "unit": "Tops/s",
                "frac": prods / (ms * 1e-3) / peak_prod, "traffic": None,
                "time": "the whole graph launch (counter reset, a prep and a propagate launch per chunk), not the "
                        "propagate kernel alone",
                "peak_source": "measured live on this GPU (bench_pipes.cu) at %.0f MHz SM clock, %d SMs"
                               % (prod_mhz, n_sm),
                "hbm_output_gbs": pairs * 36 / (ms * 1e-3) / 1e9}
    if rank == 0:
        line = {"metric": "(cos,E) pairs/s, %d parameter sets with uneven grids in one persistent CUDA-graph "
                          "launch (mixed)" % n,
                "value": world * pairs / (ms * 1e-3), "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "i32 Q1.30 chain + f32 phases + double-float eigen-solve (float out)",
                "data": "synthetic",
                "config": {"workload": "%d sets, cosines U{64..1024} in [-1,0], energies U{64..2048} over "
                                       "0.5-100 GeV, density scale U(0.97,1.03), seeds 0 (parameters) and 3 "
                                       "(grids)" % n, "pairs_per_step": pairs,
                           "l2": "outputs %.1f GB per step exceed L2" % (pairs * 36 / 1e9),
                           "launch_shape": {"te": te, "groups": groups, "cchunk": cchunk, "blocks": blocks},
                           "autotune_s": tune_s, "autotune_best_ms": tune_ms},
                "sequential": {"value": world * pairs / (seq_ms * 1e-3), "unit": "pairs/s", "ms_per_step": seq_ms,
                               "launches_per_step": 2 * n},
                "speedup_vs_sequential": seq_ms / ms, "gpu_launches": kernels_per_step * args.steps,
                "kernels_per_step": kernels_per_step, "clocks": clocks, "roofline": roofline,
                "precision": {"max_abs_dp_vs_oracle_sampled_sets": err,
                              "mean_abs_dp_vs_oracle_sampled_sets": float(np.mean(errs)),
                              "sampled": "every %d-th set, every 16th cosine and energy" % max(1, n // 8)}}
        print(json.dumps(line), flush=True)
    b.close()


def run_rates(args, world, rank, local):
    """Fused event rates on the 4096 x 4096 grid: rate_b = sum_a flux_a P(a -> b)
    histogrammed into 400 cosine x 200 energy bins inside the propagation
    kernel (nu + nubar per step), so the 2 x 604 MB of planes never leave the
    GPU.  Flux E^-2.7 with nu_e = nu_mu / 2 and no nu_tau (resident on the
    device, as in a fit).  e2e: the lists uploaded and both histograms read
    back to the host every step.  Checked against the same sums over the
    probability planes of the plane path."""
    import torch

    import cudaprob3_gb300 as cp

    torch.cuda.set_device(local)
    dev = local
    cos, en, B, nom = grid()
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    ncb, neb = 400, 200
    cb = ((np.arange(NC) * ncb) // NC).astype(np.int32)
    eb = ((np.arange(NE) * neb) // NE).astype(np.int32)
    phi = (en ** -2.7).astype(np.float32)
    flux = np.zeros((3, NC, NE), np.float32)
    flux[0] = 0.5 * phi[None, :]
    flux[1] = phi[None, :]
    props = []
    for anti in (False, True):
        p = make_prop(cp, "mixed", cos, en, B, nom, dev)
        p.set_stream(stream.cuda_stream)
        p.setRateFlux(flux, 3)
        p.setRateBins(cb, eb, ncb, neb)
        props.append((p, cp.Antineutrino if anti else cp.Neutrino))
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            for p, t in props:
                p.calculateRatesAsync(t)
        stream.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        evs = []
        sampler = ClockSampler(dev)
        sampler.start()
        for _ in range(args.steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for p, t in props:
                p.calculateRatesAsync(t)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        clocks = sampler.stop()
        barrier(world)
    ms = allmax(world, float(np.mean([a.elapsed_time(b) for a, b in evs])))
    pairs_step = 2 * NC * NE
    # e2e through the public API: lists in, histograms out, every step
    e2e_steps = max(3, min(args.steps, 20))
    hosts = [np.empty((3, ncb, neb)) for _ in props]
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for (p, t), h in zip(props, hosts):
            p.setEnergyList(en)
            p.setCosineList(cos)
            p.calculateRates(t, out=h)
    e2e_s = allmax(world, (time.perf_counter() - t0) / e2e_steps)
    # check: the same histograms from the plane path, summed on the device
    err = 0.0
    idx = torch.as_tensor((cb[:, None].astype(np.int64) * neb + eb[None, :]).ravel(), device=dev)
    fl = torch.as_tensor(flux, device=dev).double()
    for (p, t), h in zip(props, hosts):
        buf = torch.empty((9, NC, NE), dtype=torch.float32, device=dev)
        p.set_result_buffer(buf.data_ptr(), buf.numel() * 4)
        p.calculateProbabilities(t)
        P = buf.view(3, 3, NC, NE).double()
        rate = torch.einsum("acd,abcd->bcd", fl, P).reshape(3, -1)
        want = torch.zeros((3, ncb * neb), dtype=torch.float64, device=dev)
        want.index_add_(1, idx, rate)
        want = want.cpu().numpy().reshape(3, ncb, neb)
        err = max(err, float(np.abs(h - want).max() / np.abs(want).max()))
        p.set_result_buffer(0, 0)
        del buf
    if rank == 0:
        line = {"metric": "(cos,E) pairs/s propagated and histogrammed (fused event rates, mixed)",
                "value": world * pairs_step / (ms * 1e-3), "unit": "pairs/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "i32 Q1.30 chain + f32 phases + double-float eigen-solve, f32 run sums, f64 histograms",
                "data": "synthetic",
                "config": {"workload": WORKLOAD + "; rates into 400 cos x 200 E bins, flux E^-2.7, nu_e = nu_mu/2",
                           "pairs_per_step": pairs_step,
                           "l2": "flushed between steps (256 MB write outside the timed events)"},
                "e2e": {"value": world * pairs_step / e2e_s, "unit": "pairs/s",
                        "h2d_bytes_per_step": 2 * 8 * (NC + NE), "d2h_bytes_per_step": 2 * 3 * ncb * neb * 8,
                        "ms_per_step": e2e_s * 1e3},
                "gpu_launches": 2 * 2 * args.steps, "clocks": clocks,
                "precision": {"max_rel_diff_vs_plane_path": err}}
        print(json.dumps(line), flush=True)
    for p, _ in props:
        p.close()


def run_heights(args, world, rank, local):
    """The 4096 x 4096 grid (nu + nubar per step) with probabilities averaged
    over 8 production heights (10-45 km, weights of a broad hump): the chain
    runs once per pair, each height adds a phase pair and a small product.
    Reported beside the single-height time of the same grid, and checked
    against the weighted average of the oracle at each height on a strided
    subset."""
    import torch

    import cudaprob3_gb300 as cp
    import oracle

    torch.cuda.set_device(local)
    dev = local
    cos, en, B, nom = grid()
    heights = np.array([10.0, 15.0, 20.0, 25.0, 30.0, 35.0, 40.0, 45.0])
    weights = np.array([0.04, 0.10, 0.18, 0.22, 0.20, 0.14, 0.08, 0.04])
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    props, bufs = [], []
    for anti in (False, True):
        p = make_prop(cp, "mixed", cos, en, B, nom, dev)
        buf = torch.empty((9, NC, NE), dtype=torch.float32, device=dev)
        p.set_result_buffer(buf.data_ptr(), buf.numel() * 4)
        p.set_stream(stream.cuda_stream)
        props.append((p, cp.Antineutrino if anti else cp.Neutrino))
        bufs.append(buf)

    def timed(steps, warmup):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                for p, t in props:
                    p.calculateProbabilitiesAsync(t)
            stream.synchronize()
            barrier(world)
            evs = []
            for _ in range(steps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                for p, t in props:
                    p.calculateProbabilitiesAsync(t)
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize()
            barrier(world)
        return allmax(world, float(np.mean([a.elapsed_time(b) for a, b in evs])))

    single_ms = timed(max(3, min(args.steps, 20)), args.warmup)
    for p, _ in props:
        p.setProductionHeights(heights, weights)
    sampler = ClockSampler(dev)
    sampler.start()
    ms = timed(args.steps, args.warmup)
    clocks = sampler.stop()
    # parity on a strided subset: every 64th cosine and energy
    idx = np.arange(0, NC, 64)
    err = 0.0
    means = []
    for (p, t), buf in zip(props, bufs):
        p.calculateProbabilities(t)
        got = buf.cpu().numpy()[:, idx][:, :, idx].astype(np.float64)
        w = weights / weights.sum()
        want = sum(wk * oracle.calculate(cos[idx], en[idx], B.radii, B.rho_eff(), nom, float(h),
                                         t == cp.Antineutrino) for h, wk in zip(heights, w))
        err = max(err, float(np.abs(got - want).max()))
        means.append(float(np.abs(got - want).mean()))
    pairs_step = 2 * NC * NE
    if rank == 0:
        line = {"metric": "(cos,E) pairs/s with probabilities averaged over 8 production heights (mixed)",
                "value": world * pairs_step / (ms * 1e-3), "unit": "pairs/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "i32 Q1.30 chain + f32 phases + double-float eigen-solve, f32 height sums (float out)",
                "data": "synthetic",
                "config": {"workload": WORKLOAD + "; heights 10-45 km (8), weights " +
                           ",".join("%.2f" % x for x in weights), "pairs_per_step": pairs_step,
                           "l2": "flushed between steps (256 MB write outside the timed events)"},
                "single_height": {"value": world * pairs_step / (single_ms * 1e-3), "ms_per_step": single_ms},
                "cost_vs_single_height": ms / single_ms,
                "gpu_launches": 2 * 2 * args.steps, "clocks": clocks,
                "precision": {"max_abs_dp_vs_oracle_height_average_subset": err,
                              "mean_abs_dp_vs_oracle_height_average_subset": float(np.mean(means)),
                              "subset": "every 64th cosine x every 64th energy, nu and nubar"}}
        print(json.dumps(line), flush=True)
    for p, _ in props:
        p.close()


PRECISION_N = 8192


def precision_sets(local, nsets):
    """The precision workload: nsets parameter sets of seed 0 (Gaussian around
    nominal, random sign of dm32; neutrinos for even sets, antineutrinos for
    odd ones) on the 8192 x 8192 grid (cosines in [-1, 0], 0.1-1000 GeV) of the
    11-shell body.  Per set: the mixed and the FP64 kernel (CUDA events on
    their stream), max/mean |dP| of mixed against FP64 over all 67M pairs
    (on the device), and both against the oracle on every 128th cosine and
    energy (64 x 64 pairs).  Returns the summary and the per-set rows."""
    import torch

    import cudaprob3_gb300 as cp
    from cudaprob3_gb300 import grids as G
    import oracle

    n = PRECISION_N
    cos = G.linspace(-1.0, 0.0, n)
    en = G.logspace(0.1, 1000.0, n)
    B = G.PREM_12
    sets = G.draw_parameter_sets(nsets, seed=0)
    pm = make_prop(cp, "mixed", cos, en, B, G.NOMINAL, local)
    pf = make_prop(cp, "fp64", cos, en, B, G.NOMINAL, local)
    bm = torch.empty((9, n, n), dtype=torch.float32, device=local)
    bf = torch.empty((9, n, n), dtype=torch.float64, device=local)
    pm.set_result_buffer(bm.data_ptr(), bm.numel() * 4)
    pf.set_result_buffer(bf.data_ptr(), bf.numel() * 8)
    stream = torch.cuda.Stream(device=local)
    pm.set_stream(stream.cuda_stream)
    pf.set_stream(stream.cuda_stream)
    idx = np.arange(0, n, 128)
    per_set = []
    tm = []
    tf = []
    for k, ps in enumerate(sets):
        anti = bool(k % 2)
        t = cp.Antineutrino if anti else cp.Neutrino
        for p in (pm, pf):
            p.setMNSMatrix(*ps[:4])
            p.setNeutrinoMasses(*ps[4:])
        with torch.cuda.stream(stream):
            for p, acc in ((pm, tm), (pf, tf)):
                a = torch.cuda.Event(enable_timing=True)
                c = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                p.calculateProbabilitiesAsync(t)
                c.record(stream)
                c.synchronize()
                acc.append(a.elapsed_time(c))
            d = (bm.double() - bf).abs_()
            dmax, dmean = float(d.max()), float(d.mean())
            del d
        want = oracle.calculate(cos[idx], en[idx], B.radii, B.rho_eff(), tuple(ps), 22.0, anti)
        gm = bm[:, idx][:, :, idx].double().cpu().numpy()
        gf = bf[:, idx][:, :, idx].cpu().numpy()
        per_set.append({"set": k, "anti": anti, "dm32": float(ps[5]), "max_vs_fp64": dmax, "mean_vs_fp64": dmean,
                        "max_mixed_vs_oracle": float(np.abs(gm - want).max()),
                        "mean_mixed_vs_oracle": float(np.abs(gm - want).mean()),
                        "max_fp64_vs_oracle": float(np.abs(gf - want).max())})
    pm.close()
    pf.close()
    del bm, bf
    torch.cuda.empty_cache()
    pairs = n * n
    mix_ms = float(np.median(tm))
    f64_ms = float(np.median(tf))
    summary = {"workload": "8192 cos x 8192 E (0.1-1000 GeV), 11-shell PREM, %d parameter sets from seed 0 "
                           "(nu for even sets, nubar for odd; %d with dm32 < 0)" % (nsets, sum(r["dm32"] < 0 for r in per_set)),
               "oracle_subset": "every 128th cosine and energy (64 x 64) per set",
               "max_mixed_vs_fp64": max(r["max_vs_fp64"] for r in per_set),
               "max_of_set_means_mixed_vs_fp64": max(r["mean_vs_fp64"] for r in per_set),
               "mean_of_set_means_mixed_vs_fp64": float(np.mean([r["mean_vs_fp64"] for r in per_set])),
               "max_mixed_vs_oracle": max(r["max_mixed_vs_oracle"] for r in per_set),
               "max_fp64_vs_oracle": max(r["max_fp64_vs_oracle"] for r in per_set),
               "mixed_pairs_per_s": pairs / (mix_ms * 1e-3), "fp64_pairs_per_s": pairs / (f64_ms * 1e-3),
               "mixed_ms_median": mix_ms, "fp64_ms_median": f64_ms, "speedup_mixed_vs_fp64": f64_ms / mix_ms,
               "timing": "one calculation (prep + propagate) per set and form, CUDA events on its stream, median "
                         "over the sets; outputs 2.4 GB (mixed) / 4.8 GB (FP64) per calculation exceed L2"}
    return summary, per_set


def run_precision(args, world, rank, local):
    import torch

    torch.cuda.set_device(local)
    nsets = args.sets or 64
    summary, per_set = precision_sets(local, nsets)
    if rank == 0:
        line = {"metric": "per-set max/mean |dP| of the mixed kernel, 8192 x 8192, %d parameter sets" % nsets,
                "value": summary["max_mixed_vs_fp64"], "unit": "max |dP| mixed vs FP64 (all pairs)",
                "higher_is_better": False, "n_gpus": world, "data": "synthetic",
                "config": {"workload": summary["workload"], "oracle_subset": summary["oracle_subset"]},
                "summary": summary, "per_set": per_set}
        print(json.dumps(line), flush=True)


def run_gradient(args, world, rank, local):
    """400 x 200 binned Poisson log-likelihood: gradient evaluations/s (FP64
    and mixed adjoint) and the relative error of each against central finite
    differences (h = 1e-6 relative) of the FP64 oracle."""
    import torch

    from cudaprob3_gb300.loglik import PARAM_NAMES, binned_problem
    import oracle

    torch.cuda.set_device(local)
    prob = binned_problem(device_id=local)
    B = prob.body
    x0 = np.concatenate([prob.nominal, B.rhos])

    def oracle_ll(x):
        p = oracle.calculate(prob.cosines, prob.energies, B.radii, (x[6:] * B.ye) / 0.5, tuple(x[:6]), prob.height,
                             False)
        return prob.loglik(p[1], p[4])

    fd = np.zeros_like(x0)
    steps = np.zeros_like(x0)
    for k in range(x0.size):
        h = 1e-6 * abs(x0[k])
        steps[k] = h
        xp, xm = x0.copy(), x0.copy()
        xp[k] += h
        xm[k] -= h
        fd[k] = (oracle_ll(xp) - oracle_ll(xm)) / (2 * h)
    # cancellation noise of the central differences: each LL carries about
    # eps * sum_b |n_b ln(lambda_b)| + lambda_b of rounding, divided by 2h
    ll_abs = prob.loglik_abs_sum(oracle.calculate(prob.cosines, prob.energies, B.radii, (B.rhos * B.ye) / 0.5,
                                                  tuple(prob.nominal), prob.height, False))
    fd_noise = np.where(steps > 0, 2.2e-16 * ll_abs / (2 * np.where(steps > 0, steps, 1.0)), 0.0)
    # components whose central difference is good to 1e-6 relative or better
    resolved = fd_noise < 1e-6 * np.abs(fd)
    # layer counts of the bins (the library's own setDensity / maxlayers) and
    # the pair kernel's multiply-adds over all bins
    import cudaprob3_gb300 as cp
    with cp.CudaPropagatorSingle(local, prob.cosines.size, 1, precision="fp64") as h:
        h.setCosineList(prob.cosines)
        h.setDensity(B.radii, B.rhos, B.ye)
        ml = h.maxlayers()
    pair_fmas = float(ll_pair_products_per_pair(ml).sum()) * prob.energies.size
    peak = {"mixed": pipe_peak(PIPE_FFMA, local), "fp64": pipe_peak(PIPE_DFMA, local)}
    out = {}
    for precision in ("fp64", "mixed"):
        L = prob.make(device_id=local, precision=precision)
        t0 = time.perf_counter()
        for _ in range(max(3, args.warmup)):
            ll, g = L.evaluate(prob.nominal, B.rhos)
        est = (time.perf_counter() - t0) / max(3, args.warmup)
        # about 1.5 s of evaluations, so that the clock sampler (100 ms) sees the run
        n = max(20, args.steps, min(50000, int(1.5 / max(est, 1e-6))))
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.start()
        t0 = time.perf_counter()
        for _ in range(n):
            ll, g = L.evaluate(prob.nominal, B.rhos)
        dt = (time.perf_counter() - t0) / n
        clocks = sampler.stop()
        # each kernel's time from events recorded inside the graph (a second,
        # separately timed pass: the events are not part of the timed graph)
        L.set_kernel_timing(True)
        L.evaluate(prob.nominal, B.rhos)
        kt = []
        for _ in range(min(n, 200)):
            L.evaluate(prob.nominal, B.rhos)
            kt.append(L.last_kernel_ms())
        L.set_kernel_timing(False)
        prep_ms, pair_ms, layer_ms = (float(np.median([k[i] for k in kt])) for i in range(3))
        pk, pk_mhz, pk_sms = peak[precision]
        roof = {"bound": "FP32 FMA pipe" if precision == "mixed" else "FP64 pipe (DFMA)",
                "kernel": "ll_pair_kernel<%s>" % ("float" if precision == "mixed" else "double"),
                "work_per_launch": pair_fmas,
                "work_unit": "real multiply-adds of the forward chain and its adjoint per bin "
                             "(ll_pair_products_per_pair) summed over the 80,000 bins",
                "kernel_ms": pair_ms, "achieved": pair_fmas / (pair_ms * 1e-3) / 1e12, "peak": pk / 1e12,
                "unit": "T FMA/s", "frac": pair_fmas / (pair_ms * 1e-3) / pk, "traffic": None,
                "peak_source": "measured live on this GPU (bench_pipes.cu) at %.0f MHz SM clock" % pk_mhz,
                "kernels_ms": {"ll_prep_kernel": prep_ms, "ll_pair_kernel": pair_ms, "ll_layer_kernel": layer_ms},
                "prep_and_layer": "FP64, latency-bound (a few warps per SM): %d eigen-solves per evaluation in "
                                  "ll_prep_kernel, %d (energy, layer) back-propagations in ll_layer_kernel"
                                  % (prob.energies.size * (B.rhos.size + 1), prob.energies.size * (B.rhos.size + 1))}
        names = list(PARAM_NAMES) + ["rho_row%d" % i for i in range(B.rhos.size)]
        rel = np.abs(g - fd) / np.linalg.norm(fd)
        # element-wise |g_k - fd_k| / |fd_k|; a zero FD component (the zero-width
        # centre row) is compared in absolute terms
        elem = np.where(fd != 0.0, np.abs(g - fd) / np.where(fd != 0.0, np.abs(fd), 1.0), np.abs(g))
        io_up, io_down = L.io_bytes()
        out[precision] = {"evals_per_s": 1.0 / dt, "ms_per_eval": dt * 1e3, "evaluations": n, "clocks": clocks,
                          "h2d_bytes_per_eval": io_up, "d2h_bytes_per_eval": io_down,
                          "loglik": ll, "roofline": roof,
                          "max_rel_grad_error": float(elem[resolved].max()),
                          "max_rel_grad_error_note": "element-wise |g - fd| / |fd| over the components whose "
                                                     "central difference carries less than 1e-6 relative "
                                                     "cancellation noise (fd_noise_rel_per_param)",
                          "rel_grad_error_per_param": {n_: float(r) for n_, r in zip(names, elem)},
                          "max_grad_error_over_fd_norm": float(rel.max()),
                          "gradient": g.tolist()}
        L.close()
    if rank == 0:
        line = {"metric": "gradient evaluations/s, binned Poisson log-likelihood 400 cos x 200 E (adjoint)",
                "value": world * out["mixed"]["evals_per_s"], "unit": "evaluations/s", "higher_is_better": True,
                "n_gpus": world, "steps": out["mixed"]["evaluations"], "warmup": max(3, args.warmup),
                "ms_per_step": out["mixed"]["ms_per_eval"], "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 pair kernel (double-float phases) + double-float eigen-solves + f64 back-propagation",
                "data": "synthetic", "clocks": out["mixed"]["clocks"],
                "gpu_launches": 3 * out["mixed"]["evaluations"],
                "e2e": {"value": world * out["mixed"]["evals_per_s"], "unit": "evaluations/s",
                        "h2d_bytes_per_step": out["mixed"]["h2d_bytes_per_eval"],
                        "d2h_bytes_per_step": out["mixed"]["d2h_bytes_per_eval"],
                        "note": "evaluate() is host-timed end to end: the parameters go up by the graph's first "
                                "copy and the per-energy rows come back through mapped host memory"},
                "config": {"workload": "400 x 200 bins (cos [-1,0], 0.5-100 GeV log), flux E^-2.7 (nu_e = nu_mu/2), "
                                       "1e6 expected events, Poisson counts seed 1 at nominal + 1 sigma "
                                       "(theta23, dcp, dm32); gradient w.r.t. 6 parameters + 12 row densities",
                           "wall_clock": "one evaluate() = graph launch with parameter upload and gradient "
                                         "download, host-timed"},
                "roofline": out["mixed"]["roofline"],
                "fp64": out["fp64"], "mixed": out["mixed"], "finite_differences": fd.tolist(),
                "fd_noise_rel_per_param": {n_: float(v / abs(f)) if f != 0 else None for n_, v, f in
                                           zip(list(PARAM_NAMES) + ["rho_row%d" % i for i in range(B.rhos.size)],
                                               fd_noise, fd)},
                "mixed_vs_fp64_adjoint_max_rel": float(np.max(
                    np.abs(np.array(out["mixed"]["gradient"]) - np.array(out["fp64"]["gradient"])) /
                    np.maximum(np.abs(np.array(out["fp64"]["gradient"])), 1e-300)))}
        print(json.dumps(line), flush=True)


def run_profile_case(args):
    """One propagation of an n x n grid (cosines in [-1, 0], energies log-spaced
    over 0.1-1000 GeV, 11-shell body, nominal parameters), repeated, for a
    profiler: the nine planes, fused event rates into 400 x 200 bins (flux
    E^-2.7, nu_e = nu_mu / 2), planes averaged over 8 production heights
    (10-45 km), or evaluations of the 400 x 200 binned log-likelihood and its
    gradient (n does not apply).  Prints the wall time per calculation."""
    import cudaprob3_gb300 as cp
    from cudaprob3_gb300 import grids as G
    if args.profile_case == "bands":
        # one launch per crossed-shell count M: 256 cosines strictly inside the
        # band of M shells (between the M-th and (M+1)-th cosine limits of
        # the 11-shell body) x 1024 energies, so that per-pair counters of
        # the launches separate the cost of an inner layer from the fixed part
        B = G.PREM_12
        r = np.sort(B.radii)[::-1]
        lim = -np.sqrt(1.0 - (r / 6371.0) ** 2)
        lim[0] = 0.0
        en = G.logspace(0.1, 1000.0, 1024)
        for M in args.bands:
            c = np.linspace(lim[M], lim[M - 1], 258)[1:-1]
            with cp.CudaPropagatorSingle(0, c.size, en.size, precision=args.precision) as p:
                p.setEnergyList(en)
                p.setCosineList(c)
                p.setMNSMatrix(*G.NOMINAL[:4])
                p.setNeutrinoMasses(*G.NOMINAL[4:])
                p.setDensity(B.radii, B.rhos, B.ye)
                p.setProductionHeight(G.PRODUCTION_HEIGHT_KM)
                if not (p.maxlayers() == M).all():
                    raise RuntimeError("band %d: cosines outside the band" % M)
                p.calculateProbabilities(cp.Neutrino)
            print("band M=%d: %d x %d pairs" % (M, c.size, en.size), flush=True)
        return
    if args.profile_case == "gradient":
        from cudaprob3_gb300.loglik import binned_problem
        prob = binned_problem(device_id=0)
        L = prob.make(device_id=0, precision=args.precision)
        L.evaluate(prob.nominal, prob.body.rhos)
        t0 = time.perf_counter()
        for _ in range(args.repeat):
            L.evaluate(prob.nominal, prob.body.rhos)
        dt = time.perf_counter() - t0
        L.close()
        print("gradient precision=%s repeat=%d: %.3f ms per evaluation" % (args.precision, args.repeat,
                                                                           1e3 * dt / args.repeat))
        return
    n = args.n
    c = G.linspace(-1.0, 0.0, n)
    e = G.logspace(0.1, 1000.0, n)
    B = G.PREM_12
    with cp.CudaPropagatorSingle(0, n, n, precision=args.precision) as p:
        p.setEnergyList(e)
        p.setCosineList(c)
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(B.radii, B.rhos, B.ye)
        p.setProductionHeight(G.PRODUCTION_HEIGHT_KM)
        if args.profile_case == "heights":
            p.setProductionHeights(np.arange(10.0, 46.0, 5.0), [0.04, 0.10, 0.18, 0.22, 0.20, 0.14, 0.08, 0.04])
        if args.profile_case == "rates":
            phi = (e ** -2.7).astype(np.float32)
            flux = np.zeros((3, n, n), np.float32)
            flux[0] = 0.5 * phi[None, :]
            flux[1] = phi[None, :]
            p.setRateFlux(flux, 3)
            p.setRateBins((np.arange(n) * 400) // n, (np.arange(n) * 200) // n, 400, 200)
        t = cp.Antineutrino if args.anti else cp.Neutrino
        t0 = time.perf_counter()
        for _ in range(args.repeat):
            if args.profile_case == "rates":
                p.calculateRates(t)
            else:
                p.calculateProbabilities(t)
        dt = time.perf_counter() - t0
        print("n=%d precision=%s case=%s repeat=%d: %.3f ms per calculation" % (
            n, args.precision, args.profile_case, args.repeat, 1e3 * dt / args.repeat))


def main():
    args = parse()
    if args.profile_case:
        run_profile_case(args)
        return
    world, rank, local = dist_init(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        elif args.workload == "batch":
            run_batch(args, world, rank, local)
        elif args.workload == "precision":
            run_precision(args, world, rank, local)
        elif args.workload == "gradient":
            run_gradient(args, world, rank, local)
        elif args.workload == "rates":
            run_rates(args, world, rank, local)
        elif args.workload == "heights":
            run_heights(args, world, rank, local)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()

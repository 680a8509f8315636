"""Distinct handles used from distinct host threads at the same time, as the C
header allows: four threads, each with its own propagator (mixed and FP64, the
12- and 59-row bodies, so that kernels of several shared-memory sizes are
opted in from several threads at once; different grids and parameter sets),
create their handles together and calculate repeatedly; every result equals
the same configuration's result computed alone, bit for bit.  A fifth thread
makes failing calls throughout: the error message is per thread, so it reads
its own message while the others succeed.  (ctypes releases the GIL around
each foreign call, so the library is entered from the threads concurrently.)
"""
import os
import threading

import numpy as np
import pytest

from conftest import GOLDEN
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu

REPEAT = 12


def bodies():
    r59, d59 = G.read_density_file(os.path.join(GOLDEN, "models", "PREM_59layer.dat"))
    return {"prem12": G.PREM_12, "prem59": G.Body(r59, d59, np.where(r59 <= 3480.0, 0.468, 0.497))}


def configs():
    rng = np.random.default_rng(7)
    sets = G.draw_parameter_sets(4, seed=3)
    out = []
    for k, (precision, body, nc, ne) in enumerate([("mixed", "prem12", 300, 257), ("fp64", "prem59", 96, 130),
                                                    ("mixed", "prem59", 129, 200), ("fp64", "prem12", 150, 77)]):
        c = np.sort(rng.uniform(-1.0, 0.3, nc))
        e = G.logspace(0.2, 300.0, ne)
        out.append(dict(precision=precision, body=body, cos=c, en=e, params=tuple(float(x) for x in sets[k]),
                        anti=bool(k & 1)))
    return out


def run(gpu, cfg, B, repeat=1, start=None, sink=None):
    with gpu.CudaPropagatorSingle(0, cfg["cos"].size, cfg["en"].size, precision=cfg["precision"]) as p:
        if start is not None:
            start.wait()
        p.setEnergyList(cfg["en"])
        p.setCosineList(cfg["cos"])
        p.setMNSMatrix(*cfg["params"][:4])
        p.setNeutrinoMasses(*cfg["params"][4:])
        p.setDensity(B.radii, B.rhos, B.ye)
        p.setProductionHeight(20.0)
        res = None
        for _ in range(repeat):
            p.calculateProbabilities(gpu.Antineutrino if cfg["anti"] else gpu.Neutrino)
            res = p.results().copy()
            if sink is not None:
                sink.append(res)
        return res


def test_handles_on_threads_match_single_thread_results(gpu):
    B = bodies()
    cfgs = configs()
    want = [run(gpu, c, B[c["body"]]) for c in cfgs]
    start = threading.Barrier(len(cfgs) + 1)
    got = [[] for _ in cfgs]
    errors = []
    seen_msgs = []
    stop = threading.Event()

    def worker(k):
        try:
            run(gpu, cfgs[k], B[cfgs[k]["body"]], REPEAT, start, got[k])
        except Exception as exc:  # reported below
            errors.append((k, repr(exc)))

    def failing():
        # a handle without a density: every calculation fails with the
        # reference's message, on this thread only
        try:
            with gpu.CudaPropagatorSingle(0, 8, 8, precision="mixed") as p:
                p.setEnergyList(G.logspace(1, 10, 8))
                p.setCosineList(G.linspace(-1, 0, 8))
                p.setMNSMatrix(*G.NOMINAL[:4])
                p.setNeutrinoMasses(*G.NOMINAL[4:])
                p.setProductionHeight(20.0)
                start.wait()
                while not stop.is_set() or len(seen_msgs) < 50:
                    try:
                        p.calculateProbabilities(gpu.Neutrino)
                        errors.append(("failing", "calculation without a density succeeded"))
                        return
                    except gpu.CP3Error as exc:
                        seen_msgs.append(str(exc))
        except Exception as exc:
            errors.append(("failing", repr(exc)))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(len(cfgs))]
    ft = threading.Thread(target=failing)
    for t in threads + [ft]:
        t.start()
    for t in threads:
        t.join(timeout=600)
    stop.set()
    ft.join(timeout=600)
    assert not any(t.is_alive() for t in threads + [ft]), "a thread did not finish"
    assert not errors, errors
    for k, c in enumerate(cfgs):
        assert len(got[k]) == REPEAT
        for r in got[k]:
            assert np.array_equal(r, want[k]), "thread %d (%s, %s) differs from its single-thread result" % (
                k, c["precision"], c["body"])
    assert seen_msgs and all("density was not set" in m for m in seen_msgs), set(seen_msgs)

"""GPU parity: the CUDA library (through the C ABI) against the golden vectors
of the reference and against the oracle on full grids.

Tolerances (max |dP| over all nine channels):
  fp64  1e-11  (the degenerate dm21 = 0 and dm32 = 0 cases: 1e-9; the reference's
               degeneracy break leaves an eigenvalue gap of 5e-9 eV^2, and both the
               reference and this library lose accuracy as eps*|H|/gap there)
  mixed 1e-6
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_golden
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "mixed": 1e-6}


def make(cp, precision, cos, en, radii, rhos, ye, params, h=22.0):
    p = cp.CudaPropagatorSingle(0, len(cos), len(en), precision=precision)
    p.setEnergyList(en)
    p.setCosineList(cos)
    p.setMNSMatrix(*params[:4])
    p.setNeutrinoMasses(*params[4:])
    p.setDensity(radii, rhos, ye)
    p.setProductionHeight(h)
    return p


def run(cp, precision, cos, en, radii, rhos, ye, params, h=22.0, anti=False):
    with make(cp, precision, cos, en, radii, rhos, ye, params, h) as p:
        p.calculateProbabilities(cp.Antineutrino if anti else cp.Neutrino)
        return p.results().astype(np.float64)


def tol_for(name, precision):
    if precision == "fp64" and ("dm12_zero" in name or "dm23_zero" in name):
        return 1e-9
    return TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", golden_cases())
def test_golden_and_oracle(gpu, precision, name):
    g = load_golden(name)
    params = tuple(g["params"])
    anti = bool(g["anti"])
    got = run(gpu, precision, g["cosines"], g["energies"], g["radii"], g["rhos"], g["ye"], params,
              float(g["height_km"]), anti)
    tol = tol_for(name, precision)
    sub = got[:, g["idx_c"]][:, :, g["idx_e"]]
    err_golden = np.abs(sub - g["probs"]).max()
    want = oracle.calculate(g["cosines"], g["energies"], g["radii"], (g["rhos"] * g["ye"]) / 0.5, params,
                            float(g["height_km"]), anti)
    err_oracle = np.abs(got - want).max()
    assert err_golden <= tol, "golden max|dP| = %.3g" % err_golden
    assert err_oracle <= tol, "oracle max|dP| = %.3g" % err_oracle


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_unitarity(gpu, precision):
    c = G.linspace(-1, 1, 97)
    e = G.logspace(0.1, 1000, 131)
    for anti in (False, True):
        p = run(gpu, precision, c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL, anti=anti)
        s = p.reshape(3, 3, len(c), len(e))
        t = 1e-12 if precision == "fp64" else 1e-6
        assert np.abs(s.sum(axis=0) - 1).max() < t
        assert np.abs(s.sum(axis=1) - 1).max() < t


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nc,ne", [(1, 1), (1, 37), (3, 1), (5, 129), (130, 7)])
def test_ragged_sizes(gpu, precision, nc, ne):
    c = G.linspace(-1, 0, nc) if nc > 1 else np.array([-0.7])
    e = G.logspace(0.2, 200, ne) if ne > 1 else np.array([3.0])
    got = run(gpu, precision, c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL)
    want = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL)
    assert got.shape == (9, nc, ne)
    assert np.abs(got - want).max() <= TOL[precision]


@pytest.mark.parametrize("precision,anti", [("fp64", False), ("mixed", False), ("mixed", True)])
def test_low_energies(gpu, precision, anti):
    """0.1 MeV - 0.1 GeV: phases of up to 1e5 turns across the Earth, where the
    double-float remainder of the mixed kernel's phase product reaches the
    table step (its Taylor correction still holds down to 0.1 MeV)."""
    c = G.linspace(-1, 0, 64)
    e = G.logspace(1e-4, 0.1, 40)
    got = run(gpu, precision, c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL, anti=anti)
    want = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, anti)
    assert np.abs(got - want).max() <= (1e-9 if precision == "fp64" else TOL[precision])


def test_empty_grid(gpu):
    with gpu.CudaPropagatorSingle(0, 0, 16) as p:
        p.setEnergyList(G.logspace(1, 10, 16))
        p.setCosineList([])
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(G.PREM_4.radii, G.PREM_4.rhos)
        p.setProductionHeight(22.0)
        p.calculateProbabilities(gpu.Neutrino)
        assert p.results().shape == (9, 0, 16)
        assert p.last_launch_count() == 0


def test_error_behaviour(gpu):
    cp = gpu
    with cp.CudaPropagatorSingle(0, 4, 5) as p:
        with pytest.raises(cp.CP3Error, match="must set cosine list before production height"):
            p.setProductionHeight(22.0)
        with pytest.raises(cp.CP3Error, match="not created for this number of energy nodes"):
            p.setEnergyList([1.0, 2.0])
        with pytest.raises(cp.CP3Error, match="not created for this number of cosine nodes"):
            p.setCosineList([-1.0])
        with pytest.raises(cp.CP3Error, match="radii order messed up"):
            p.setDensity([0.0, 3000.0, 2000.0], [1.0, 1.0, 1.0])
        with pytest.raises(cp.CP3Error, match="vectors must not be empty"):
            p.setDensity([], [])
        with pytest.raises(cp.CP3Error, match="rhos.size"):
            p.setDensity([0.0, 1.0], [1.0])
        p.setCosineList([-1.0, -0.5, 0.0, 0.5])
        p.setEnergyList([1.0, 2.0, 3.0, 4.0, 5.0])
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(G.PREM_4.radii, G.PREM_4.rhos)
        with pytest.raises(cp.CP3Error, match="production height was not set"):
            p.calculateProbabilities(cp.Neutrino)
        p.setProductionHeight(22.0)
        p.calculateProbabilities(cp.Neutrino)
        with pytest.raises(cp.CP3Error, match="Invalid indices"):
            p.getProbability(4, 0, cp.ProbType.e_e)
        with pytest.raises(cp.CP3Error, match="Invalid indices"):
            p.getProbability(0, 5, cp.ProbType.e_e)
        with pytest.raises(cp.CP3Error, match="energies must be finite and positive"):
            p.setEnergyList([1.0, 2.0, 0.0, 4.0, 5.0])
    with pytest.raises(cp.CP3Error, match="is not available"):
        cp.CudaPropagatorSingle(99, 4, 4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_get_probability_matches_planes(gpu, precision):
    c = G.linspace(-1, 0, 11)
    e = G.logspace(0.5, 100, 13)
    with make(gpu, precision, c, e, G.PREM_4.radii, G.PREM_4.rhos, G.PREM_4.ye, G.NOMINAL) as p:
        p.calculateProbabilities(gpu.Neutrino)
        planes = p.results()
        for (ic, ie, t) in [(0, 0, 0), (10, 12, 8), (5, 7, 4), (3, 2, 3)]:
            assert p.getProbability(ic, ie, gpu.ProbType(t)) == float(planes[t, ic, ie])
        # a new calculation invalidates the host copy
        p.calculateProbabilities(gpu.Antineutrino)
        anti = p.results()
        assert p.getProbability(5, 7, gpu.ProbType.m_e) == float(anti[3, 5, 7])
        assert not np.array_equal(planes, anti)


def test_density_from_file(gpu):
    c = G.linspace(-1, 0, 9)
    e = G.logspace(0.5, 100, 9)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "prem4.dat")
        with open(path, "w") as f:
            for r, rho in zip(G.PREM_4.radii, G.PREM_4.rhos):
                f.write("%.17g %.17g\n" % (r, rho))
        with make(gpu, "fp64", c, e, G.PREM_4.radii, G.PREM_4.rhos, None, G.NOMINAL) as p:
            p.calculateProbabilities(gpu.Neutrino)
            a = p.results()
            p.setDensityFromFile(path)
            p.calculateProbabilities(gpu.Neutrino)
            b = p.results()
            with pytest.raises(gpu.CP3Error, match="could not open density file"):
                p.setDensityFromFile(os.path.join(d, "missing.dat"))
    assert np.array_equal(a, b)


def test_external_buffer_and_stream(gpu):
    torch = pytest.importorskip("torch")
    c = G.linspace(-1, 0, 64)
    e = G.logspace(0.1, 1000, 96)
    with make(gpu, "mixed", c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL) as p:
        p.calculateProbabilities(gpu.Neutrino)
        own = p.results()
        buf = torch.zeros((9, 64, 96), dtype=torch.float32, device="cuda:0")
        s = torch.cuda.Stream()
        p.set_stream(s.cuda_stream)
        p.set_result_buffer(buf.data_ptr(), buf.numel() * 4)
        p.calculateProbabilitiesAsync(gpu.Neutrino)
        p.waitForCompletion()
        assert np.array_equal(buf.cpu().numpy(), own)
        p.set_result_buffer(0, 0)
        p.set_stream(0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_host_result_buffer_zero_copy(gpu, precision):
    """Kernel stores straight into page-locked host memory: same bits as the
    device buffer, getProbability reads it, pageable memory is refused."""
    torch = pytest.importorskip("torch")
    c = G.linspace(-1, 0, 80)
    e = G.logspace(0.1, 1000, 112)
    dt = torch.float32 if precision == "mixed" else torch.float64
    with make(gpu, precision, c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL) as p:
        p.calculateProbabilities(gpu.Antineutrino)
        own = p.results()
        host = torch.full((9, 80, 112), -1.0, dtype=dt).pin_memory()
        p.set_host_result_buffer(host.data_ptr(), host.numel() * host.element_size())
        p.calculateProbabilities(gpu.Antineutrino)
        assert np.array_equal(host.numpy(), own)
        assert p.getProbability(17, 33, gpu.ProbType.m_e) == float(own[3, 17, 33])
        with pytest.raises(gpu.CP3Error):
            p.set_host_result_buffer(host.data_ptr(), 16)
        pageable = np.empty(9 * 80 * 112, dtype=own.dtype)
        with pytest.raises(gpu.CP3Error, match="page-locked"):
            p.set_host_result_buffer(pageable.ctypes.data, pageable.nbytes)
        p.set_host_result_buffer(0, 0)
        p.calculateProbabilities(gpu.Neutrino)
        assert not np.array_equal(p.results(), own)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_host_completion(gpu, precision):
    """The kernel stores the 2x2 block into host memory, the host derives the
    other five planes: the stored planes are the kernel's bits, the derived
    ones within a few ulp of the device completion (1e-15 FP64, 3e-7 mixed),
    rows and columns sum to one."""
    torch = pytest.importorskip("torch")
    c = G.linspace(-1, 1, 96)
    e = G.logspace(0.1, 1000, 144)
    dt = torch.float32 if precision == "mixed" else torch.float64
    with make(gpu, precision, c, e, G.PREM_12.radii, G.PREM_12.rhos, G.PREM_12.ye, G.NOMINAL) as p:
        p.calculateProbabilities(gpu.Neutrino)
        own = p.results()
        host = torch.full((9, 96, 144), -1.0, dtype=dt).pin_memory()
        p.set_host_result_buffer(host.data_ptr(), host.numel() * host.element_size())
        p.set_host_completion(True)
        p.calculateProbabilitiesAsync(gpu.Neutrino)
        p.waitForCompletion()
        got = host.numpy()
        for t in (0, 1, 3, 4):
            assert np.array_equal(got[t], own[t])
        tol = 3e-7 if precision == "mixed" else 1e-15
        assert np.abs(got.astype(np.float64) - own).max() <= tol
        s = got.astype(np.float64).reshape(3, 3, 96, 144)
        assert np.abs(s.sum(axis=0) - 1).max() <= 4 * tol and np.abs(s.sum(axis=1) - 1).max() <= 4 * tol
        # getProbability of a derived plane after a synchronous calculation
        host.fill_(-1.0)
        p.calculateProbabilities(gpu.Antineutrino)
        assert p.getProbability(40, 70, gpu.ProbType.t_t) == float(host.numpy()[8, 40, 70])
        assert host.numpy().min() >= 0.0
        # off again: every plane from the kernel
        p.set_host_completion(False)
        p.calculateProbabilities(gpu.Neutrino)
        assert np.array_equal(host.numpy(), own)
        p.set_host_result_buffer(0, 0)


def test_configs1_scale_mixed_vs_fp64(gpu):
    """4096 x 4096 grid, 0.1-1000 GeV, 11-shell body: the mixed kernel against
    the FP64 kernel on every pair (device-side comparison) and against the
    oracle on a strided 256 x 256 subset, for both neutrino types."""
    torch = pytest.importorskip("torch")
    n = 4096
    c = G.linspace(-1, 0, n)
    e = G.logspace(0.1, 1000, n)
    B = G.PREM_12
    pf = make(gpu, "fp64", c, e, B.radii, B.rhos, B.ye, G.NOMINAL)
    pm = make(gpu, "mixed", c, e, B.radii, B.rhos, B.ye, G.NOMINAL)
    bf = torch.empty((9, n, n), dtype=torch.float64, device="cuda:0")
    bm = torch.empty((9, n, n), dtype=torch.float32, device="cuda:0")
    pf.set_result_buffer(bf.data_ptr(), bf.numel() * 8)
    pm.set_result_buffer(bm.data_ptr(), bm.numel() * 4)
    idx = np.arange(0, n, 16)
    for anti in (False, True):
        t = gpu.Antineutrino if anti else gpu.Neutrino
        pf.calculateProbabilities(t)
        pm.calculateProbabilities(t)
        ds = bm.double() - bf
        d = ds.abs()
        assert float(d.max()) <= 1e-6
        assert float(d.mean()) <= 1e-7
        # no systematic drift per channel from the chain's floor rounding
        # (measured <= 5.5e-9; the float32 output rounding alone averages 6e-9)
        assert float(ds.view(9, -1).mean(1).abs().max()) <= 2e-8
        want = oracle.calculate(c[idx], e[idx], B.radii, B.rho_eff(), G.NOMINAL, 22.0, anti)
        gf = bf.cpu().numpy()[:, idx][:, :, idx]
        assert np.abs(gf - want).max() <= 1e-11
        s = bm.view(3, 3, n, n).double()
        assert float((s.sum(0) - 1).abs().max()) <= 1e-6
    pf.close()
    pm.close()


def test_configs2_scale_parameter_sets(gpu):
    """The precision workload at full size: 8192 x 8192 grid (0.1-1000 GeV,
    11-shell body) for sets 0-3 of the 64 Gaussian parameter sets of seed 0
    (sets 0, 1 and 3 have dm32 < 0), neutrinos and antineutrinos.  Mixed
    against FP64 on every one of the 67M pairs, on the device: max |dP| <= 1e-6
    (the bar), mean <= 1e-7, per-channel mean signed error <= 2e-8; FP64
    against the oracle on every 128th cosine and energy: <= 1e-11."""
    torch = pytest.importorskip("torch")
    n = 8192
    c = G.linspace(-1, 0, n)
    e = G.logspace(0.1, 1000, n)
    B = G.PREM_12
    sets = G.draw_parameter_sets(64, seed=0)[:4]
    assert (sets[:, 5] < 0).sum() == 3
    pf = make(gpu, "fp64", c, e, B.radii, B.rhos, B.ye, G.NOMINAL)
    pm = make(gpu, "mixed", c, e, B.radii, B.rhos, B.ye, G.NOMINAL)
    bf = torch.empty((9, n, n), dtype=torch.float64, device="cuda:0")
    bm = torch.empty((9, n, n), dtype=torch.float32, device="cuda:0")
    pf.set_result_buffer(bf.data_ptr(), bf.numel() * 8)
    pm.set_result_buffer(bm.data_ptr(), bm.numel() * 4)
    idx = np.arange(0, n, 128)
    for ps in sets:
        for p in (pf, pm):
            p.setMNSMatrix(*ps[:4])
            p.setNeutrinoMasses(*ps[4:])
        for anti in (False, True):
            t = gpu.Antineutrino if anti else gpu.Neutrino
            pf.calculateProbabilities(t)
            pm.calculateProbabilities(t)
            ds = bm.double() - bf
            chan = ds.view(9, -1).mean(1).abs().max()
            ds.abs_()
            assert float(ds.max()) <= 1e-6, (tuple(ps), anti, float(ds.max()))
            assert float(ds.mean()) <= 1e-7
            assert float(chan) <= 2e-8
            del ds
            want = oracle.calculate(c[idx], e[idx], B.radii, B.rho_eff(), tuple(ps), 22.0, anti)
            gf = bf[:, idx][:, :, idx].cpu().numpy()
            assert np.abs(gf - want).max() <= 1e-11
    pf.close()
    pm.close()
    del bf, bm
    torch.cuda.empty_cache()


@pytest.mark.parametrize("which", ["dm21_zero", "dm32_zero"])
def test_degenerate_masses_at_scale(gpu, which):
    """The degeneracy breaks of setNeutrinoMasses (propagator.hpp:233-236: an
    eigenvalue gap of 5e-9 eV^2) on the 4096 x 4096 grid, both neutrino types:
    mixed against FP64 on every pair (max |dP| <= 1e-6, mean <= 1e-7), FP64
    against the oracle on every 64th cosine and energy (1e-9, the degenerate
    cases' tolerance: the reference itself loses accuracy as eps*|H|/gap)."""
    torch = pytest.importorskip("torch")
    n = 4096
    c = G.linspace(-1, 0, n)
    e = G.logspace(0.1, 1000, n)
    B = G.PREM_12
    params = list(G.NOMINAL)
    params[4 if which == "dm21_zero" else 5] = 0.0
    params = tuple(params)
    pf = make(gpu, "fp64", c, e, B.radii, B.rhos, B.ye, params)
    pm = make(gpu, "mixed", c, e, B.radii, B.rhos, B.ye, params)
    bf = torch.empty((9, n, n), dtype=torch.float64, device="cuda:0")
    bm = torch.empty((9, n, n), dtype=torch.float32, device="cuda:0")
    pf.set_result_buffer(bf.data_ptr(), bf.numel() * 8)
    pm.set_result_buffer(bm.data_ptr(), bm.numel() * 4)
    idx = np.arange(0, n, 64)
    for anti in (False, True):
        t = gpu.Antineutrino if anti else gpu.Neutrino
        pf.calculateProbabilities(t)
        pm.calculateProbabilities(t)
        d = (bm.double() - bf).abs_()
        assert float(d.max()) <= 1e-6 and float(d.mean()) <= 1e-7, (which, anti, float(d.max()))
        del d
        want = oracle.calculate(c[idx], e[idx], B.radii, B.rho_eff(), params, 22.0, anti)
        assert np.abs(bf[:, idx][:, :, idx].cpu().numpy() - want).max() <= 1e-9
    pf.close()
    pm.close()
    del bf, bm
    torch.cuda.empty_cache()


def test_pipe_peaks_are_plausible(gpu):
    """The roofline denominators of bench.py (bench_pipes.cu, a library of its
    own): each probe's rate per SM and per clock, at the SM clock the probe
    recorded over its own run, lies within 0.8-1.05 of GB300's nominal rate --
    32 integer products (mul.wide.s32), 128 FP32 FMAs and 2 FP64 FMAs per
    clock per SM (1.25 TFLOP/s FP64 at 2.07 GHz on 152 SMs) -- so a probe 20 %
    off fails."""
    import ctypes

    lib = ctypes.CDLL(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "libbench_pipes.so"))
    lib.bench_pipe_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    lib.bench_pipe_peak.restype = ctypes.c_int
    nominal = {0: 32.0, 1: 128.0, 2: 2.0}
    for pipe, per_clk in nominal.items():
        ops, mhz, sms = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        assert lib.bench_pipe_peak(0, pipe, ctypes.byref(ops), ctypes.byref(mhz), ctypes.byref(sms)) == 0
        assert 500.0 < mhz.value < 2500.0 and sms.value > 0, (mhz.value, sms.value)
        rate = ops.value / (sms.value * mhz.value * 1e6)
        assert 0.8 * per_clk <= rate <= 1.05 * per_clk, (pipe, rate, per_clk)

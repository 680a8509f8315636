"""Edge cases of the propagation against the oracle, both precisions:
  * the largest body the handle takes (64 rows: 65 layers, so that the mixed
    kernel halves its energy tile and cosine chunk to fit shared memory) and
    the 65-row body it refuses;
  * energies up to 1e6 GeV, where the matter term dominates and the phases
    are small (the reference's own FP64 roots lose digits there: the oracle's
    rows and columns sum to one only to ~6e-11, so FP64 is held to 2e-10
    against it and to 1e-12 on its own unitarity);
  * cosines exactly on the shell boundaries coslimit = -sqrt(1 - r^2/R^2)
    (a trajectory tangent to a shell) and one ulp to either side, where the
    layer count and the chord lengths switch (propagator.hpp:149-158,
    301-307; physics.hpp:555-580);
  * no mixing (all angles zero: the eigenvectors are the axes, P = identity),
    maximal mixing, and a body of vacuum rows (zero density);
  * random bodies and parameters;
  * a grid whose planes pass 2^31 elements.
Tolerances: FP64 1e-11 (2e-10 at the highest energies), mixed 1e-6."""
import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "mixed": 1e-6}
R_EARTH = 6371.0


def run(gpu, precision, cos, en, radii, rhos, ye, params, anti=False, h=22.0):
    with gpu.CudaPropagatorSingle(0, len(cos), len(en), precision=precision) as p:
        p.setEnergyList(en)
        p.setCosineList(cos)
        p.setMNSMatrix(*params[:4])
        p.setNeutrinoMasses(*params[4:])
        p.setDensity(radii, rhos, ye)
        p.setProductionHeight(h)
        p.calculateProbabilities(gpu.Antineutrino if anti else gpu.Neutrino)
        return p.results().astype(np.float64)


def body_64():
    rng = np.random.default_rng(5)
    radii = np.concatenate([[0.0], np.sort(rng.uniform(10.0, R_EARTH - 10.0, 62)), [R_EARTH]])
    rhos = np.sort(rng.uniform(1.0, 13.0, 64))[::-1].copy()
    ye = np.where(radii <= 3480.0, 0.468, 0.497)
    return G.Body(radii, rhos, ye)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("anti", [False, True])
def test_largest_body(gpu, precision, anti):
    B = body_64()
    c, e = G.linspace(-1, 0.2, 67), G.logspace(0.1, 200, 75)
    got = run(gpu, precision, c, e, B.radii, B.rhos, B.ye, G.NOMINAL, anti)
    want = oracle.calculate(c, e, B.radii, B.rho_eff(), G.NOMINAL, 22.0, anti)
    assert np.abs(got - want).max() <= TOL[precision]


def test_body_above_the_row_limit_is_refused(gpu):
    B = body_64()
    radii = np.concatenate([[0.0], np.sort(np.append(B.radii[1:-1], 3000.5)), [R_EARTH]])
    assert radii.size == 65
    with gpu.CudaPropagatorSingle(0, 4, 4, precision="mixed") as p:
        with pytest.raises(gpu.CP3Error, match="more than 64 rows"):
            p.setDensity(radii, np.ones(65))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_highest_energies(gpu, precision):
    B = G.PREM_12
    c, e = G.linspace(-1, 0.2, 41), G.logspace(1e2, 1e6, 37)
    for anti in (False, True):
        got = run(gpu, precision, c, e, B.radii, B.rhos, B.ye, G.NOMINAL, anti)
        want = oracle.calculate(c, e, B.radii, B.rho_eff(), G.NOMINAL, 22.0, anti)
        tol = 2e-10 if precision == "fp64" else TOL[precision]
        assert np.abs(got - want).max() <= tol
        s = got.reshape(3, 3, c.size, e.size)
        unit = 1e-12 if precision == "fp64" else 1e-6
        assert np.abs(s.sum(axis=0) - 1).max() <= unit and np.abs(s.sum(axis=1) - 1).max() <= unit


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cosines_on_shell_boundaries(gpu, precision):
    B = G.PREM_12
    # the host's cosine limits (propagator.hpp:149-158), and one ulp either side
    lim = -np.sqrt(1.0 - (B.radii * B.radii) / (R_EARTH * R_EARTH))
    lim = lim[(lim > -1.0) & (lim < 0.0)]
    c = np.clip(np.concatenate([lim, np.nextafter(lim, -2.0), np.nextafter(lim, 2.0), [-1.0, 0.0]]), -1.0, 1.0)
    e = G.logspace(0.3, 80, 23)
    # the layer counts follow the oracle's (strict c < coslimit)
    with gpu.CudaPropagatorSingle(0, c.size, e.size, precision=precision) as p:
        p.setEnergyList(e)
        p.setCosineList(c)
        p.setDensity(B.radii, B.rhos, B.ye)
        assert np.array_equal(p.maxlayers(), oracle.maxlayers(c, B.radii))
    for anti in (False, True):
        got = run(gpu, precision, c, e, B.radii, B.rhos, B.ye, G.NOMINAL, anti)
        want = oracle.calculate(c, e, B.radii, B.rho_eff(), G.NOMINAL, 22.0, anti)
        assert np.abs(got - want).max() <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["no_mixing", "maximal_mixing", "vacuum_body"])
def test_parameter_and_body_extremes(gpu, precision, case):
    B = G.PREM_12
    params, rhos = G.NOMINAL, B.rhos
    if case == "no_mixing":
        params = (0.0, 0.0, 0.0, 0.0) + tuple(G.NOMINAL[4:])
    elif case == "maximal_mixing":
        params = (np.pi / 4, np.pi / 4, np.pi / 4, np.pi / 2) + tuple(G.NOMINAL[4:])
    else:
        rhos = np.zeros_like(B.rhos)
    c, e = G.linspace(-1, 1, 45), G.logspace(0.1, 300, 39)
    for anti in (False, True):
        got = run(gpu, precision, c, e, B.radii, rhos, B.ye, params, anti)
        want = oracle.calculate(c, e, B.radii, rhos * B.ye / 0.5, params, 22.0, anti)
        assert np.abs(got - want).max() <= TOL[precision], (case, anti)
        if case == "no_mixing":
            s = got.reshape(3, 3, c.size, e.size)
            for k in range(3):
                assert np.abs(s[k, k] - 1.0).max() <= TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_output_beyond_32_bit_element_indices(gpu, precision):
    """A 16384 x 16384 grid: its nine planes hold 2.4e9 elements, more than a
    32-bit index reaches, so every offset of the writeback and of the host
    copy must be 64-bit.  Pairs spread over the grid up to the far corner of
    the last plane against the oracle, and over every pair on the device:
    the rows of |S|^2 (planes in*3 + out, out = 0..2) sum to one.  For the
    mixed planes, getProbability at the far corner through the handle's own
    buffer and its host copy."""
    torch = pytest.importorskip("torch")
    n = 16384
    c, e = G.linspace(-1, 0, n), G.logspace(0.1, 1000, n)
    B = G.PREM_12
    dt = torch.float32 if precision == "mixed" else torch.float64
    buf = torch.empty((9, n, n), dtype=dt, device="cuda:0")
    assert buf.numel() > 2**31
    with gpu.CudaPropagatorSingle(0, n, n, precision=precision) as p:
        p.setEnergyList(e)
        p.setCosineList(c)
        p.setMNSMatrix(*G.NOMINAL[:4])
        p.setNeutrinoMasses(*G.NOMINAL[4:])
        p.setDensity(B.radii, B.rhos, B.ye)
        p.setProductionHeight(22.0)
        p.set_result_buffer(buf.data_ptr(), buf.numel() * buf.element_size())
        p.calculateProbabilities(gpu.Neutrino)
        torch.cuda.synchronize()
    idx = np.r_[0:n:2048, n - 1]
    want = oracle.calculate(c[idx], e[idx], B.radii, B.rho_eff(), G.NOMINAL, 22.0, False)
    got = buf[:, idx][:, :, idx].double().cpu().numpy()
    assert np.abs(got - want).max() <= TOL[precision]
    rows = buf.view(3, 3, n, n).sum(dim=1, dtype=torch.float64)
    assert float((rows - 1.0).abs().max()) <= (1e-6 if precision == "mixed" else 1e-12)
    del rows, buf
    torch.cuda.empty_cache()
    if precision == "mixed":
        with gpu.CudaPropagatorSingle(0, n, n, precision=precision) as p:
            p.setEnergyList(e)
            p.setCosineList(c)
            p.setMNSMatrix(*G.NOMINAL[:4])
            p.setNeutrinoMasses(*G.NOMINAL[4:])
            p.setDensity(B.radii, B.rhos, B.ye)
            p.setProductionHeight(22.0)
            p.calculateProbabilities(gpu.Neutrino)
            for t in (0, 4, 8):
                assert abs(p.getProbability(n - 1, n - 1, t) - want[t, -1, -1]) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_random_bodies(gpu, precision):
    """Random bodies (1-20 rows, outermost radius 6371 km, the rest strictly
    decreasing at random spacings, with or without a radius-0 row; densities
    0-15 g/cm^3, electron fractions 0.40-0.60, rows given outside-in or
    inside-out), random oscillation parameters of either ordering, both
    neutrino types, cosines over [-1, 1]: both kernels against the oracle."""
    rng = np.random.default_rng(11)
    c, e = G.linspace(-1, 1, 23), G.logspace(0.2, 200.0, 29)
    for trial in range(8):
        n = int(rng.integers(1, 21))
        inner = np.sort(rng.uniform(0.0, R_EARTH, size=n - 1))[::-1]
        radii = np.concatenate([[R_EARTH], inner])
        if n > 1 and rng.random() < 0.5:
            radii[-1] = 0.0
        if len(np.unique(radii)) != n:
            continue
        rhos = rng.uniform(0.0, 15.0, size=n)
        ye = rng.uniform(0.40, 0.60, size=n)
        if rng.random() < 0.5:  # inside-out order
            radii, rhos, ye = radii[::-1].copy(), rhos[::-1].copy(), ye[::-1].copy()
        params = tuple(G.draw_parameter_sets(1, seed=100 + trial)[0])
        anti = bool(trial & 1)
        got = run(gpu, precision, c, e, radii, rhos, ye, params, anti)
        want = oracle.calculate(c, e, radii, rhos * ye / 0.5, params, 22.0, anti)
        assert np.abs(got - want).max() <= TOL[precision], (trial, n, precision)

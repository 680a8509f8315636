"""The oracle (C restatement of the reference's CpuPropagator) against the
golden vectors produced by the reference itself, plus physics invariants."""
import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_golden
from cudaprob3_gb300 import grids as G


@pytest.mark.parametrize("name", golden_cases())
def test_port_matches_reference_goldens(name):
    g = load_golden(name)
    rho_eff = (g["rhos"] * g["ye"]) / 0.5
    p = oracle.calculate(g["cosines"], g["energies"], g["radii"], rho_eff, tuple(g["params"]),
                         float(g["height_km"]), bool(g["anti"]))
    sub = p[:, g["idx_c"]][:, :, g["idx_e"]]
    # bit-identical on the machine that produced the fixtures; libm may differ
    # by an ulp elsewhere
    assert np.abs(sub - g["probs"]).max() <= 1e-12


def test_reference_probe_values():
    """P(mu -> mu) of the reference's CpuPropagator<double> on the 4-shell body
    (neutrinos, 256 x 256 grid) at cos = -1, E = 0.5 GeV and cos = 0,
    E = 100 GeV, as a run of the reference printed them."""
    g = load_golden("prem4_256_ye05")
    ic = list(g["idx_c"])
    ie = list(g["idx_e"])
    pm = g["probs"][4]
    assert pm[ic.index(0), ie.index(0)] == pytest.approx(0.6946042163303086, abs=1e-13)
    assert pm[ic.index(255), ie.index(255)] == pytest.approx(0.9997167925019199, abs=1e-13)


@pytest.mark.parametrize("anti", [False, True])
def test_unitarity(anti):
    c = G.linspace(-1, 1, 33)
    e = G.logspace(0.1, 1000, 29)
    p = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, anti)
    s = p.reshape(3, 3, len(c), len(e))
    assert np.abs(s.sum(axis=0) - 1).max() < 1e-12
    assert np.abs(s.sum(axis=1) - 1).max() < 1e-12


def test_vacuum_limit_matches_analytic_formula():
    # zero density everywhere: three-flavour vacuum oscillation over the path
    t12, t13, t23, dcp, dm21, dm32 = G.NOMINAL
    c = G.linspace(-1, 1, 9)
    e = G.logspace(0.5, 50, 7)
    p = oracle.calculate(c, e, [0.0, 6371.0], [0.0, 0.0], G.NOMINAL, 22.0, False)
    s12, s13, s23 = np.sin([t12, t13, t23])
    c12, c13, c23 = np.cos([t12, t13, t23])
    ed = np.exp(1j * dcp)
    U = np.array([[c12 * c13, s12 * c13, s13 / ed],
                  [-s12 * c23 - c12 * s23 * s13 * ed, c12 * c23 - s12 * s23 * s13 * ed, s23 * c13],
                  [s12 * s23 - c12 * c23 * s13 * ed, -c12 * s23 - s12 * c23 * s13 * ed, c23 * c13]])
    m = np.array([0.0, dm21, dm21 + dm32])
    R = 6371e5
    for ic, cz in enumerate(c):
        L = (np.sqrt((R + 22e5) ** 2 - R * R * (1 - cz * cz)) - R * cz) / 1e5
        for ie, E in enumerate(e):
            A = U @ np.diag(np.exp(-1j * 2.534 * m * L / E)) @ U.conj().T
            want = (np.abs(A.T) ** 2).reshape(9)
            assert np.abs(p[:, ic, ie] - want).max() < 1e-11


def test_upgoing_crosses_only_atmosphere():
    c = np.array([0.0, 0.3, 1.0])
    e = G.logspace(0.5, 50, 5)
    a = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, False)
    b = oracle.calculate(c, e, G.PREM_4.radii, G.PREM_4.rho_eff(), G.NOMINAL, 22.0, False)
    assert np.array_equal(a, b)


def test_maxlayers_counts_cosine_limits():
    c = np.array([-1.0, -0.999, -0.9, -0.5, -0.1, -1e-9, 0.0, 0.5])
    m = oracle.maxlayers(c, G.PREM_4.radii)
    assert list(m) == [4, 4, 3, 2, 1, 1, 0, 0]


def test_float_port_runs_and_is_far_from_fp64():
    """The reference's FP32 path: documents its error against FP64."""
    c = G.linspace(-1, 0, 64)
    e = G.logspace(0.1, 1000, 64)
    p64 = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, False)
    p32 = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, False,
                           precision="f32")
    err = np.abs(p32.astype(np.float64) - p64).max()
    assert 1e-6 < err < 1e-1


@pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")
def test_port_bit_identical_to_reference_build():
    c = G.linspace(-1, 0.4, 31)
    e = G.logspace(0.1, 1000, 27)
    for prec in ("f64", "f32"):
        for anti in (False, True):
            a = oracle.calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, anti,
                                 precision=prec)
            b = oracle.ref_calculate(c, e, G.PREM_12.radii, G.PREM_12.rho_eff(), G.NOMINAL, 22.0, anti,
                                     precision=prec)
            assert np.array_equal(a, b)


def test_oracle_rejects_unsorted_radii():
    with pytest.raises(RuntimeError):
        oracle.calculate([-1.0], [1.0], [0.0, 3000.0, 2000.0], [1.0, 1.0, 1.0], G.NOMINAL)

import numpy as np
import pytest

from cudaprob3_gb300 import grids as G


def test_linspace_endpoints_and_accumulation():
    x = G.linspace(-1.0, 0.0, 256)
    assert x[0] == -1.0 and x[-1] == 0.0
    step = 1.0 / 255
    acc = -1.0
    for i in range(255):
        assert x[i] == acc
        acc += step


def test_logspace_endpoints():
    x = G.logspace(0.1, 1000.0, 4096)
    assert x[0] == 0.1 and x[-1] == 1000.0
    assert np.all(np.diff(x) > 0)
    assert np.allclose(np.diff(np.log(x[1:-1])), np.log(1e4) / 4095, rtol=1e-9)


def test_zero_points_rejected():
    with pytest.raises(ValueError):
        G.linspace(0, 1, 0)


def test_parameter_draws_are_seeded():
    a = G.draw_parameter_sets(64, seed=0)
    b = G.draw_parameter_sets(64, seed=0)
    assert np.array_equal(a, b)
    assert set(np.sign(a[:, 5])) == {-1.0, 1.0}


def test_bodies():
    assert G.PREM_12.radii.size == 12 and G.PREM_12.radii[0] == 0.0
    assert np.allclose(G.PREM_4.rho_eff() * 0.5, G.PREM_4.rhos * G.PREM_4.ye)

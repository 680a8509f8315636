"""Adjoint gradient of the binned Poisson log-likelihood against central
finite differences (h = 1e-6 relative) of the FP64 oracle.

Tolerances: LL to 1e-9 relative; FP64 gradient to 1e-4 relative of the
gradient's norm per component (the finite differences themselves are good to
about 1e-6 of the norm); mixed gradient to 1e-3.  The inert radius-0 row of
the body has an exactly zero gradient.
"""
import numpy as np
import pytest

import oracle
from cudaprob3_gb300 import grids as G

pytestmark = pytest.mark.gpu


def oracle_ll(prob, params, rhos):
    B = prob.body
    p = oracle.calculate(prob.cosines, prob.energies, B.radii, (np.asarray(rhos) * B.ye) / 0.5, tuple(params),
                         prob.height, False)
    return prob.loglik(p[1], p[4])


def fd_gradient(prob, params, rhos, h=1e-6):
    x0 = np.concatenate([params, rhos])
    g = np.zeros_like(x0)
    for k in range(x0.size):
        step = h * abs(x0[k]) if x0[k] != 0 else h
        xp, xm = x0.copy(), x0.copy()
        xp[k] += step
        xm[k] -= step
        g[k] = (oracle_ll(prob, xp[:6], xp[6:]) - oracle_ll(prob, xm[:6], xm[6:])) / (2 * step)
    return g


@pytest.fixture(scope="module")
def problem(gpu):
    from cudaprob3_gb300.loglik import binned_problem
    return binned_problem(n_cos=64, n_en=40)


@pytest.fixture(scope="module")
def fd(problem):
    return fd_gradient(problem, problem.nominal, problem.body.rhos)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-4), ("mixed", 1e-3)])
def test_gradient_matches_finite_differences(problem, fd, precision, tol):
    with problem.make(precision=precision) as L:
        ll, g = L.evaluate(problem.nominal, problem.body.rhos)
    want_ll = oracle_ll(problem, problem.nominal, problem.body.rhos)
    assert abs(ll - want_ll) <= (1e-9 if precision == "fp64" else 1e-6) * abs(want_ll) + 1e-6
    scale = np.linalg.norm(fd)
    err = np.abs(g - fd) / scale
    assert err.max() <= tol, "per-component error / |grad|: %s" % np.array2string(err, precision=2)
    # the radius-0 row of the 12-row body is never crossed
    assert g[6 + 0] == 0.0 and fd[6 + 0] == 0.0


def _prem59():
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "prem59.npz"))
    return G.Body(d["radii"], d["rhos"], d["ye"])


@pytest.mark.parametrize("body_name", ["prem4", "prem59"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-4), ("mixed", 1e-3)])
def test_gradient_other_bodies_ragged_grid(gpu, body_name, precision, tol):
    """4 and 60 density rows (the layer kernel's packing: 6 energies per block
    at 5 layers, one per block at 61), 50 x 30 bins (a partial cosine chunk
    and a partial energy tile)."""
    from cudaprob3_gb300.loglik import binned_problem
    body = G.PREM_4 if body_name == "prem4" else _prem59()
    prob = binned_problem(n_cos=50, n_en=30, body=body)
    fd = fd_gradient(prob, prob.nominal, body.rhos)
    with prob.make(precision=precision) as L:
        ll, g = L.evaluate(prob.nominal, body.rhos)
    want_ll = oracle_ll(prob, prob.nominal, body.rhos)
    assert abs(ll - want_ll) <= (1e-9 if precision == "fp64" else 1e-6) * abs(want_ll) + 1e-6
    assert g.shape == (6 + body.rhos.size,)
    err = np.abs(g - fd) / np.linalg.norm(fd)
    assert err.max() <= tol, "per-component error / |grad|: %s" % np.array2string(err, precision=2)


def test_gradient_is_deterministic_and_moves_with_parameters(problem):
    with problem.make(precision="fp64") as L:
        a = L.evaluate(problem.nominal, problem.body.rhos)
        b = L.evaluate(problem.nominal, problem.body.rhos)
        c = L.evaluate(problem.observed_at, problem.body.rhos)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
    assert c[0] > a[0]  # the observed point fits its own data better


def test_loglik_io_bytes(problem):
    with problem.make(precision="mixed") as L:
        up, down = L.io_bytes()
    rows = len(problem.body.radii)
    # one row per energy back (its log-likelihood term and 6 + rows gradient
    # terms, doubles); the parameter block and one rho*Ye per layer up
    assert down == 8 * len(problem.energies) * (7 + rows)
    assert 8 * (rows + 1) < up < 4096


def test_loglik_errors(gpu):
    from cudaprob3_gb300 import CP3Error
    from cudaprob3_gb300.loglik import LogLikelihood
    with LogLikelihood(0, 4, 5) as L:
        with pytest.raises(CP3Error, match="must be set"):
            L.evaluate(np.array(G.NOMINAL), np.ones(5))
        # the body goes through the single-grid handle's checks (propagator.hpp:117-161)
        with pytest.raises(CP3Error, match="radii order messed up"):
            L.set_body([0.0, 3000.0, 2000.0])
        with pytest.raises(CP3Error, match="must be finite"):
            L.set_body([0.0, np.nan])
        with pytest.raises(CP3Error, match="electron fractions"):
            L.set_body([0.0, 6371.0], [0.5, -0.1])
        with pytest.raises(CP3Error, match="more than 64 rows"):
            L.set_body(np.linspace(0.0, 6371.0, 65))

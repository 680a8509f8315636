"""The algebra behind the propagate kernels, checked in FP64 numpy on random
layers (no GPU, no oracle): the reference multiplies the layer propagators in
the order A_1..A_{M-1} A_M A_{M-1}..A_1 A_0 (physics.hpp:645-677); the
kernels use

  * a real basis: A_l = W V_l D_l V_l^T W^dagger with V_l real orthogonal
    (det +1), D_l diagonal phases, W = R23 diag(1, 1, e^{i delta});
  * transpose symmetry: S_r = V_1 (Y^T D_M Y) T_0 D_0 V_0^T with
    Y = T_{M-1} D_{M-1} ... T_1 D_1 and T_l = V_{l+1}^T V_l;
  * two columns: the third column of the unitary Y is det(Y) conj(c0 x c1);
  * the 2x2 block: |S|^2 is doubly stochastic, so the block of rows and
    columns (e, mu) fixes the other five probabilities.
"""
import numpy as np
import pytest


def rotation(i, j, a, n=3):
    r = np.eye(n)
    r[i, i] = r[j, j] = np.cos(a)
    r[i, j] = np.sin(a)
    r[j, i] = -np.sin(a)
    return r


def layer(rng, h0):
    """Eigen-basis (det +1) and phases of H = h0 - fac e0 e0^T over a length."""
    fac = rng.uniform(0.0, 3.0)
    h = h0.copy()
    h[0, 0] -= fac
    m, v = np.linalg.eigh(h)
    if np.linalg.det(v) < 0:
        v[:, 2] = -v[:, 2]
    length = rng.uniform(0.1, 5.0)
    d = np.exp(-1j * (m - m[0]) * length)  # phases relative to the first eigenvalue
    return v, d


def case(seed, M):
    rng = np.random.default_rng(seed)
    t12, t13, t23, dcp = rng.uniform(0.1, 1.4, 3).tolist() + [rng.uniform(0, 2 * np.pi)]
    o = rotation(0, 2, t13) @ rotation(0, 1, t12)  # O = R13 R12 (real)
    h0 = o @ np.diag([0.0, rng.uniform(0.1, 1.0), rng.uniform(1.0, 5.0)]) @ o.T
    w = rotation(1, 2, t23) @ np.diag([1.0, 1.0, np.exp(1j * dcp)])
    layers = [layer(rng, h0) for _ in range(M + 1)]  # 0 = atmosphere, 1..M shells
    return w, layers


def reference_order(w, layers, M):
    """S_f = A_1 .. A_{M-1} A_M A_{M-1} .. A_1 A_0, A_l = W V_l D_l V_l^T W^dagger."""
    A = [w @ v @ np.diag(d) @ v.T @ w.conj().T for v, d in layers]
    s = A[0]
    for l in range(1, M):
        s = A[l] @ s
    if M >= 1:
        s = A[M] @ s
    for l in range(M - 1, 0, -1):
        s = A[l] @ s
    return s


def restructured(w, layers, M):
    """S_f = W V_1 (Y^T D_M Y) T_0 D_0 V_0^T W^dagger (M >= 1), Y = T_{M-1} D_{M-1}..T_1 D_1."""
    V = [v for v, _ in layers]
    D = [np.diag(d) for _, d in layers]
    T = [V[l + 1].T @ V[l] for l in range(M)]
    y = np.eye(3, dtype=complex)
    for l in range(1, M):
        y = T[l] @ D[l] @ y
    G = y.T @ D[M] @ y
    return w @ V[1] @ G @ T[0] @ D[0] @ V[0].T @ w.conj().T, y


@pytest.mark.parametrize("M", [1, 2, 3, 6, 12])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_transpose_symmetry(seed, M):
    w, layers = case(seed, M)
    ref = reference_order(w, layers, M)
    s, _ = restructured(w, layers, M)
    assert np.max(np.abs(s - ref)) < 1e-12
    assert np.max(np.abs(s @ s.conj().T - np.eye(3))) < 1e-12


@pytest.mark.parametrize("M", [2, 5, 12])
def test_third_column_from_two(M):
    w, layers = case(7, M)
    _, y = restructured(w, layers, M)
    c0, c1 = y[:, 0], y[:, 1]
    rebuilt = np.linalg.det(y) * np.conj(np.cross(c0, c1))
    assert np.max(np.abs(rebuilt - y[:, 2])) < 1e-12
    # det Y is the product of the layers' phase determinants (det T_l = 1)
    phase = np.prod([np.prod(d) for _, d in layers[1:M]])
    assert abs(np.linalg.det(y) - phase) < 1e-12


@pytest.mark.parametrize("seed", [3, 4])
def test_probabilities_from_the_two_by_two_block(seed):
    w, layers = case(seed, 6)
    s, _ = restructured(w, layers, 6)
    p = np.abs(s) ** 2  # p[out][in]
    q00, q01, q10, q11 = p[0, 0], p[0, 1], p[1, 0], p[1, 1]
    full = np.array([[q00, q01, 1 - q00 - q01],
                     [q10, q11, 1 - q10 - q11],
                     [1 - q00 - q10, 1 - q01 - q11, q00 + q01 + q10 + q11 - 1]])
    assert np.max(np.abs(full - p)) < 1e-12

"""Edge cases of the GPU path against the oracle (complex128, 1e-12).

Angles on the branch points of the scaled rotation forms, an empty
observable, QAOA with no layers, linearity in an unnormalised start state,
QAOA observables with non-classical terms (expectation only, as the
reference), the largest observable the observable pass takes, and the
term-count limit."""
import numpy as np
import pytest

from conftest import obs_dict, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _mc(n, L, axes, angles, kind, q0, q1, w, **kw):
    from qradient_gb300 import McClean

    return McClean(n, obs_dict(n, np.array(kind), np.array(q0), np.array(q1), np.array(w)), L,
                   axes=np.asarray(axes), angles=np.asarray(angles, dtype=np.float64), **kw)


def test_angles_on_the_form_branch_points():
    """theta in {0, +-pi/2, pi, 3pi/2, 2pi, -pi, 4pi}: cos(theta/2) or
    sin(theta/2) vanish or tie, which is where the scaled forms switch."""
    n, L = 9, 4
    grid = np.array([0.0, np.pi / 2, -np.pi / 2, np.pi, 1.5 * np.pi, 2 * np.pi, -np.pi, 4 * np.pi])
    rng = np.random.default_rng(5)
    axes = rng.integers(0, 3, (L, n))
    angles = grid[rng.integers(0, grid.size, (L, n))]
    kind, q0, q1, w = [3, 0, 1, 2], [0, 3, 5, 8], [1, 3, 5, 8], [1.0, 0.4, -0.3, 0.25]
    E0, g0 = O.mcclean_grad(n, axes, angles, O.Terms(kind, q0, q1, w))
    for mode in ("history", "uncompute"):
        E, g = _mc(n, L, axes, angles, kind, q0, q1, w, grad_mode=mode).grad_run()
        assert abs(E - E0) <= TOL
        assert np.max(np.abs(g - g0)) <= TOL * max(1.0, np.max(np.abs(g0)))


def test_empty_observable():
    from qradient_gb300 import McClean

    n, L = 6, 3
    rng = np.random.default_rng(2)
    c = McClean(n, {}, L, axes=rng.integers(0, 3, (L, n)), angles=rng.uniform(0, 6, (L, n)))
    E, g = c.grad_run()
    assert E == 0.0 and g.shape == (L, n) and np.all(g == 0.0)
    assert c.run_expec_val() == 0.0


def test_qaoa_without_layers():
    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    n = 8
    edges = random_regular_edges(3, n, 4)
    q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), 0)
    E, g = q.grad_run([], [])
    terms = O.Terms([3] * len(edges), [a for a, b in edges], [b for a, b in edges], [1.0] * len(edges))
    assert abs(E - O.qaoa_run(n, np.zeros(0), np.zeros(0), terms)) <= TOL
    assert g.shape == (0, 2)


def test_start_state_linearity():
    """E and the gradient are quadratic in the start state: 3 ini gives 9x."""
    n, L = 7, 3
    rng = np.random.default_rng(8)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    v /= np.linalg.norm(v)
    kind, q0, q1, w = [3, 0], [0, 2], [1, 2], [1.0, -0.5]
    c = _mc(n, L, axes, angles, kind, q0, q1, w)
    E1, g1 = c.grad_run(ini_state=v)
    E3, g3 = c.grad_run(ini_state=3 * v)
    assert abs(E3 - 9 * E1) <= 1e-11 * max(1.0, abs(E1))
    assert rel_err(g3, 9 * g1) <= TOL
    E0, g0 = O.mcclean_grad(n, axes, angles, O.Terms(kind, q0, q1, w), ini=v)
    assert abs(E1 - E0) <= TOL and rel_err(g1, g0) <= TOL


def test_qaoa_non_classical_terms_enter_the_expectation_only():
    from qradient_gb300 import Qaoa

    n, p = 8, 2
    edges = [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (5, 6), (6, 7), (0, 7)]
    kind = [3] * len(edges) + [0, 1]
    q0 = [a for a, b in edges] + [2, 5]
    q1 = [b for a, b in edges] + [2, 5]
    w = [1.0] * len(edges) + [0.5, -0.25]
    rng = np.random.default_rng(3)
    betas, gammas = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    with pytest.warns(UserWarning):
        q = Qaoa(n, obs_dict(n, np.array(kind), np.array(q0), np.array(q1), np.array(w)), p)
    E = q.run_expec_val(betas, gammas)
    assert abs(E - O.qaoa_run(n, betas, gammas, O.Terms(kind, q0, q1, w))) <= TOL
    # the gradient follows the classical part (qaoa.py:56-57)
    Eg, g = q.grad_run(betas, gammas)
    Ec, gc = O.qaoa_grad(n, betas, gammas, O.Terms(kind[:len(edges)], q0[:len(edges)], q1[:len(edges)],
                                                   w[:len(edges)]))
    assert rel_err(g, gc) <= TOL


def test_largest_observable():
    """Every single-qubit and every ZZ term of 16 qubits (256 terms, several
    weight runs) in one observable pass."""
    n, L = 16, 2
    rng = np.random.default_rng(13)
    kind, q0, q1, w = [], [], [], []
    for k in (0, 1, 2):
        for q in range(n):
            kind.append(k), q0.append(q), q1.append(q), w.append(float(rng.choice([0.5, -1.0, 0.25])))
    for i in range(n):
        for j in range(i + 1, n):
            kind.append(3), q0.append(i), q1.append(j), w.append(float(rng.choice([1.0, -0.5, 2.0])))
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    E0, g0 = O.mcclean_grad(n, axes, angles, O.Terms(kind, q0, q1, w))
    E, g = _mc(n, L, axes, angles, kind, q0, q1, w).grad_run()
    assert abs(E - E0) <= TOL * max(1.0, abs(E0))
    assert rel_err(g, g0) <= TOL


def test_term_count_limit_is_an_error_not_a_fault():
    from qradient_gb300 import McClean, _lib

    n = 30
    zz = np.full((n, n), None)
    for i in range(n):
        for j in range(i + 1, n):
            zz[i, j] = 1.0  # 435 terms, above the 400 one pass takes
    c = McClean(n, {"zz": zz}, 1, axes=np.zeros((1, n), dtype=int), angles=np.zeros((1, n)))
    with pytest.raises(_lib.QgradError):
        c.native()


@pytest.mark.parametrize("dtype,tol,tiles", [("complex128", 1e-12, (0, 12, 5)), ("complex64", 2e-5, (0, 13, 6))])
def test_dense_diagonal_observable(dtype, tol, tiles):
    """Every ZZ pair and every Z term of 14 qubits, weights drawn from a few
    values (runs of equal weights inside the observable pass's term subsets),
    through the per-tile term sums (default tiles), the per-element term loop
    (13-bit complex64 tiles) and small tiles."""
    n, L = 14, 3
    rng = np.random.default_rng(21)
    kind, q0, q1, w = [], [], [], []
    for q in range(n):
        kind.append(2), q0.append(q), q1.append(q), w.append(float(rng.choice([0.5, -1.0, 0.25])))
    for i in range(n):
        for j in range(i + 1, n):
            kind.append(3), q0.append(i), q1.append(j), w.append(float(rng.choice([1.0, -0.5, 2.0, 0.75])))
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    E0, g0 = O.mcclean_grad(n, axes, angles, O.Terms(kind, q0, q1, w))
    c = _mc(n, L, axes, angles, kind, q0, q1, w, dtype=dtype)
    for t in tiles:
        c.set_tuning(t, 0, 0)
        E, g = c.grad_run()
        assert abs(E - E0) <= tol * max(1.0, abs(E0)), (t, E, E0)
        assert rel_err(g, g0) <= tol, (t, rel_err(g, g0))
        assert abs(c.run_expec_val() - E0) <= tol * max(1.0, abs(E0))

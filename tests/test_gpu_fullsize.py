"""Full-size properties (n = 24..30), where the CPU oracle is too slow:
central finite differences of run_expec_val, history == uncompute, forward
E == grad_run E, complex64 against complex128 (error stated)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _chain(n, L, seed, dtype="complex128", mode="auto"):
    from qradient_gb300 import McClean

    rng = np.random.default_rng(seed)
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    return McClean(n, {"zz": zz}, L, axes=rng.integers(0, 3, (L, n)), angles=rng.uniform(0, 2 * np.pi, (L, n)),
                   dtype=dtype, grad_mode=mode)


def _fd(c, i, q, h=1e-5):
    a = np.array(c.angles, copy=True)
    p = a.copy()
    p[i, q] += h
    c.angles = p
    ep = c.run_expec_val()
    p[i, q] -= 2 * h
    c.angles = p
    em = c.run_expec_val()
    c.angles = a
    return (ep - em) / (2 * h)


def test_n24_L50_history_uncompute_fd_and_c64():
    c = _chain(24, 50, 24, mode="history")
    E, g = c.grad_run()
    assert abs(c.run_expec_val() - E) <= 1e-12
    cu = _chain(24, 50, 24, mode="uncompute")
    Eu, gu = cu.grad_run()
    assert abs(Eu - E) <= 1e-12 and rel_err(gu, g) <= 1e-12
    for (i, q) in ((0, 0), (25, 11), (49, 23)):
        assert abs(_fd(c, i, q) - g[i, q]) <= 1e-8, (i, q)
    c64 = _chain(24, 50, 24, dtype="complex64")
    E64, g64 = c64.grad_run()
    err = rel_err(g64, g)
    print("n=24 L=50: complex64 vs complex128 |dE| = %.2e, normwise gradient error %.2e, max entry error %.2e" %
          (abs(E64 - E), err, np.max(np.abs(g64 - g))))
    assert abs(E64 - E) <= 1e-4 and err <= 1e-4


def test_n28_and_n30_uncompute_fd():
    for n, L in ((28, 4), (30, 2)):
        c = _chain(n, L, n, mode="uncompute")
        E, g = c.grad_run()
        assert abs(c.run_expec_val() - E) <= 1e-12
        assert abs(_fd(c, L - 1, n // 2) - g[L - 1, n // 2]) <= 1e-8
        c._native.release_workspaces()

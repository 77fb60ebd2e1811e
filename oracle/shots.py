"""numpy restatement of the projector shot estimator.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` to check the device Pauli
expectations and projector shots.  The ``qradient_gb300`` product never
imports this module.

``sample_expec_val`` (``qradient/circuit_logic/base.py:22-33``) measures each
observable term P_k through its +1 projector (``Projector``,
``qradient/physical_components/observable.py:126-177``): a shot is +w_k with
probability p_k = ||Pi_+ psi||^2 and -w_k otherwise, and the estimate is the
sum over terms of the shot means.  p_k = (1 + <psi|P_k|psi>) / 2, so the
count of + outcomes in s shots is Binomial(s, p_k).
"""
import numpy as np

X, Y, Z, ZZ = 0, 1, 2, 3


def pauli_expectation(vec, n, kind, q0, q1=None):
    """<psi|P|psi> for one term; qubit q is index bit n - 1 - q."""
    x = np.arange(vec.size)
    b0 = n - 1 - int(q0)
    if kind in (Z, ZZ):
        par = (x >> b0) & 1
        if kind == ZZ:
            par ^= (x >> (n - 1 - int(q1))) & 1
        return float(np.sum(np.abs(vec) ** 2 * (1 - 2 * par)))
    x0 = x[((x >> b0) & 1) == 0]
    z = np.sum(np.conj(vec[x0]) * vec[x0 | (1 << b0)])
    return float(2 * z.real) if kind == X else float(2 * z.imag)


def pauli_expectations(vec, n, kind, q0, q1):
    return np.array([pauli_expectation(vec, n, k, a, b) for k, a, b in zip(kind, q0, q1)])


def p_plus(expectations):
    """Probability of the +1 outcome, base.py:26 (prob of the projector)."""
    return np.clip(0.5 * (1.0 + np.asarray(expectations)), 0.0, 1.0)


def estimate_std(expectations, weights, shots):
    """Standard deviation of the shot estimate sum_k w_k (2 c_k / s - 1)."""
    e = np.asarray(expectations)
    return np.sqrt(np.sum(np.asarray(weights) ** 2 * (1.0 - e ** 2)) / shots)

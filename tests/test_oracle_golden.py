"""The CPU oracle (oracle/qg_oracle.c) against the reference's golden vectors.

The goldens come from the reference's own circuit_logic run through
tests/golden/make_golden.py; pinning the oracle to them lets the GPU tests
use the oracle at sizes and settings the goldens do not cover."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

TOL = 1e-12


def _terms(c):
    return O.Terms(c["kind"], c["q0"], c["q1"], c["w"])


@pytest.mark.parametrize("which", ["small", "large"])
def test_mcclean_grad_matches_reference(golden, which):
    for m in golden.cases("mcclean"):
        if (m["n"] >= 16) != (which == "large"):
            continue
        c = golden.case("mcclean", m["name"])
        ent = O.ENT_CZ if m["ladder"] == "cz" else O.ENT_CNOT
        E, g = O.mcclean_grad(m["n"], c["axes"], c["angles"], _terms(c), entangler=ent, ini=c.get("ini"))
        assert abs(E - float(c["e_grad"])) <= TOL * max(1.0, abs(float(c["e_grad"]))), m["name"]
        assert rel_err(g, c["grad"]) <= TOL, (m["name"], rel_err(g, c["grad"]))


def test_mcclean_run_matches_reference(golden):
    for m in golden.cases("mcclean"):
        if m["n"] > 14:
            continue
        c = golden.case("mcclean", m["name"])
        ent = O.ENT_CZ if m["ladder"] == "cz" else O.ENT_CNOT
        E, st = O.mcclean_run(m["n"], c["axes"], c["angles"], _terms(c), entangler=ent, ini=c.get("ini"),
                              want_state=True)
        assert abs(E - float(c["e_run"])) <= TOL, m["name"]
        if "state" in c:
            assert np.max(np.abs(st - c["state"])) <= 1e-13, m["name"]


def test_qaoa_matches_reference(golden):
    for m in golden.cases("qaoa"):
        c = golden.case("qaoa", m["name"])
        t = _terms(c)
        E, g = O.qaoa_grad(m["n"], c["betas"], c["gammas"], t, ini=c.get("ini"))
        assert abs(E - float(c["e_grad"])) <= TOL * max(1.0, abs(float(c["e_grad"]))), m["name"]
        assert rel_err(g, c["grad"]) <= TOL, (m["name"], rel_err(g, c["grad"]))
        Er, st = O.qaoa_run(m["n"], c["betas"], c["gammas"], t, ini=c.get("ini"), want_state=True)
        assert abs(Er - float(c["e_run"])) <= TOL * max(1.0, abs(float(c["e_run"]))), m["name"]
        if "state" in c:
            assert np.max(np.abs(st - c["state"])) <= 1e-13, m["name"]


def test_maxcut_table_bit_exact(golden):
    for m in golden.cases("qaoa"):
        c = golden.case("qaoa", m["name"])
        if "cost_table" not in c:
            continue
        t = O.maxcut_table(m["n"], c["edges"])
        assert np.array_equal(t, c["cost_table"]), m["name"]


def test_ladder_is_a_permutation_and_inverse():
    n = 7
    rng = np.random.default_rng(3)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    w = O.entangle(n, v, O.ENT_CNOT)
    assert np.allclose(np.sort(np.abs(w)), np.sort(np.abs(v)))
    back = O.entangle(n, w, O.ENT_CNOT, inverse=True)
    assert np.array_equal(back, v)
    cz = O.entangle(n, O.entangle(n, v, O.ENT_CZ), O.ENT_CZ)
    assert np.array_equal(cz, v)


def test_finite_differences_on_oracle():
    """The oracle's adjoint gradient against central differences of its run."""
    n, L = 6, 3
    rng = np.random.default_rng(7)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    t = O.Terms([3, 0, 1], [0, 2, 4], [1, 2, 4], [1.0, 0.4, -0.3])
    for ent, place in [(O.ENT_CNOT, 0), (O.ENT_CZ, 1), (O.ENT_CNOT, 1)]:
        _, g = O.mcclean_grad(n, axes, angles, t, entangler=ent, placement=place)
        h = 1e-5
        fd = np.zeros_like(g)
        for i in range(L):
            for q in range(n):
                a = angles.copy()
                a[i, q] += h
                ep = O.mcclean_run(n, axes, a, t, entangler=ent, placement=place)
                a[i, q] -= 2 * h
                em = O.mcclean_run(n, axes, a, t, entangler=ent, placement=place)
                fd[i, q] = (ep - em) / (2 * h)
        assert np.max(np.abs(fd - g)) < 1e-8


def test_uncompute_mode_matches_history_and_reference(golden):
    """The oracle's uncompute mode (one psi taken backwards, used where the
    L+1 stored states do not fit in host memory) against its history mode
    and the reference's goldens, for every entangler and placement."""
    for m in golden.cases("mcclean"):
        if m["n"] > 14:
            continue
        c = golden.case("mcclean", m["name"])
        ent = O.ENT_CZ if m["ladder"] == "cz" else O.ENT_CNOT
        E, g = O.mcclean_grad(m["n"], c["axes"], c["angles"], _terms(c), entangler=ent, ini=c.get("ini"),
                              uncompute=True)
        assert abs(E - float(c["e_grad"])) <= TOL * max(1.0, abs(float(c["e_grad"]))), m["name"]
        assert rel_err(g, c["grad"]) <= TOL, (m["name"], rel_err(g, c["grad"]))
    n, L = 11, 7
    rng = np.random.default_rng(11)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    t = O.Terms([3, 3, 0, 1, 2], [0, 4, 2, 9, 5], [1, 10, 2, 9, 5], [1.0, -0.5, 0.4, 0.3, 0.7])
    for ent in (O.ENT_NONE, O.ENT_CNOT, O.ENT_CZ):
        for place in (O.PLACE_BEFORE, O.PLACE_AFTER):
            Eh, gh = O.mcclean_grad(n, axes, angles, t, entangler=ent, placement=place)
            Eu, gu = O.mcclean_grad(n, axes, angles, t, entangler=ent, placement=place, uncompute=True)
            assert abs(Eu - Eh) <= TOL and rel_err(gu, gh) <= TOL, (ent, place, rel_err(gu, gh))
    for m in golden.cases("qaoa"):
        c = golden.case("qaoa", m["name"])
        E, g = O.qaoa_grad(m["n"], c["betas"], c["gammas"], _terms(c), ini=c.get("ini"), uncompute=True)
        assert abs(E - float(c["e_grad"])) <= TOL * max(1.0, abs(float(c["e_grad"]))), m["name"]
        assert rel_err(g, c["grad"]) <= TOL, (m["name"], rel_err(g, c["grad"]))


def test_ladders_match_reference():
    """The oracle's open and periodic CNOT ladders, and their inverses,
    against the reference's own ladder matrices (State.load_cnot_ladder,
    state.py:209-241) applied to seeded random states."""
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ladder.npz"))
    assert bool(z["odd_n_raises"])
    for n in (2, 4, 6, 8, 10):
        for kind, ent in (("open", O.ENT_CNOT), ("periodic", O.ENT_CNOT_PERIODIC)):
            tag = "n%d/%s/" % (n, kind)
            v = z[tag + "in"]
            assert np.array_equal(O.entangle(n, v, ent), z[tag + "stack0"]), tag
            assert np.array_equal(O.entangle(n, v, ent, inverse=True), z[tag + "stack1"]), tag
    with pytest.raises(ValueError):
        O.entangle(5, np.ones(32), O.ENT_CNOT_PERIODIC)


def test_periodic_ladder_gradient_against_finite_differences():
    n, L = 6, 3
    rng = np.random.default_rng(17)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    t = O.Terms([3, 3, 0], [0, 2, 5], [1, 5, 5], [1.0, 0.7, 0.4])
    for place in (O.PLACE_BEFORE, O.PLACE_AFTER):
        _, g = O.mcclean_grad(n, axes, angles, t, entangler=O.ENT_CNOT_PERIODIC, placement=place)
        h = 1e-5
        for i, q in ((0, 0), (1, 5), (2, 3)):
            a = angles.copy()
            a[i, q] += h
            ep = O.mcclean_run(n, axes, a, t, entangler=O.ENT_CNOT_PERIODIC, placement=place)
            a[i, q] -= 2 * h
            em = O.mcclean_run(n, axes, a, t, entangler=O.ENT_CNOT_PERIODIC, placement=place)
            assert abs((ep - em) / (2 * h) - g[i, q]) < 1e-8

"""GPU parity: the native kernels (through the drop-in classes and the C ABI)
against the reference's golden vectors and the CPU oracle.

Tolerances: complex128 normwise 1e-12 (||g - g_ref||_inf / ||g_ref||_inf)
and |E - E_ref| <= 1e-12; complex64 errors are reported against the FP64
oracle and bounded by 1e-4 relative."""
import numpy as np
import pytest

from conftest import obs_dict, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 1e-4


def _mcclean(n, L, c, ladder="cnot", placement="before", dtype="complex128", grad_mode="auto"):
    from qradient_gb300 import McClean

    obs = obs_dict(n, c["kind"], c["q0"], c["q1"], c["w"])
    return McClean(n, obs, L, axes=np.asarray(c["axes"], dtype=np.int64), angles=np.asarray(c["angles"]),
                   entangler=ladder, placement=placement, dtype=dtype, grad_mode=grad_mode)


@pytest.mark.parametrize("mode", ["history", "uncompute"])
def test_mcclean_golden_c128(golden, mode):
    for m in golden.cases("mcclean"):
        c = golden.case("mcclean", m["name"])
        circ = _mcclean(m["n"], m["L"], c, ladder=m["ladder"], grad_mode=mode)
        E, g = circ.grad_run(ini_state=c.get("ini"))
        assert abs(E - float(c["e_grad"])) <= TOL128, (m["name"], E, float(c["e_grad"]))
        assert rel_err(g, c["grad"]) <= TOL128, (m["name"], rel_err(g, c["grad"]))
        Er = circ.run_expec_val(ini_state=c.get("ini"))
        assert abs(Er - float(c["e_run"])) <= TOL128, m["name"]
        if "state" in c:
            assert np.max(np.abs(circ.state.vec - c["state"])) <= 1e-13, m["name"]


def test_mcclean_golden_c64_error_stated(golden):
    worst_e, worst_g = 0.0, 0.0
    for m in golden.cases("mcclean"):
        c = golden.case("mcclean", m["name"])
        circ = _mcclean(m["n"], m["L"], c, ladder=m["ladder"], dtype="complex64")
        E, g = circ.grad_run(ini_state=c.get("ini"))
        worst_e = max(worst_e, abs(E - float(c["e_grad"])))
        worst_g = max(worst_g, rel_err(g, c["grad"]))
    print("complex64 vs FP64 reference: max |dE| = %.3e, max normwise grad error = %.3e" % (worst_e, worst_g))
    assert worst_e <= TOL64 and worst_g <= TOL64


@pytest.mark.parametrize("mode", ["history", "uncompute"])
def test_qaoa_golden_c128(golden, mode):
    from qradient_gb300 import Qaoa

    for m in golden.cases("qaoa"):
        c = golden.case("qaoa", m["name"])
        obs = obs_dict(m["n"], c["kind"], c["q0"], c["q1"], c["w"])
        circ = Qaoa(m["n"], obs, m["p"], grad_mode=mode)
        E, g = circ.grad_run(c["betas"], c["gammas"], ini_state=c.get("ini"))
        assert abs(E - float(c["e_grad"])) <= TOL128 * max(1, abs(float(c["e_grad"]))), m["name"]
        assert rel_err(g, c["grad"]) <= TOL128, (m["name"], rel_err(g, c["grad"]))
        Er = circ.run_expec_val(c["betas"], c["gammas"], ini_state=c.get("ini"))
        assert abs(Er - float(c["e_run"])) <= TOL128 * max(1, abs(float(c["e_run"]))), m["name"]
        if "state" in c:
            assert np.max(np.abs(circ.state.vec - c["state"])) <= 1e-13, m["name"]
        if "cost_table" in c:
            assert np.array_equal(circ.classical_ham().astype(np.int64), c["cost_table"].astype(np.int64))


@pytest.mark.parametrize("n,L,ladder,placement,seed", [
    (3, 2, "cz", "after", 1),
    (9, 3, "cnot", "after", 2),
    (13, 4, "cz", "before", 3),
    (14, 3, "cnot", "before", 4),
    (15, 3, "cnot", "after", 5),
    (17, 2, "cz", "after", 6),
    (18, 2, "cnot", "before", 7),
])
def test_mcclean_vs_oracle(n, L, ladder, placement, seed):
    """Random sizes (crossing the one-tile / multi-sweep boundary), both
    entanglers and placements, Pauli-sum observables with X/Y terms."""
    rng = np.random.default_rng(seed)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    kind = [3, 0, 1, 2, 3]
    q0 = [0, n - 1, n // 2, 1 % n, 1]
    q1 = [1, n - 1, n // 2, 1 % n, n - 1]
    w = [1.0, 0.3, -0.45, 0.2, 0.7]
    if n < 3:
        kind, q0, q1, w = kind[:1], q0[:1], q1[:1], w[:1]
    c = {"axes": axes, "angles": angles, "kind": np.array(kind), "q0": np.array(q0), "q1": np.array(q1),
         "w": np.array(w)}
    t = O.Terms(kind, q0, q1, w)
    ent = O.ENT_CZ if ladder == "cz" else O.ENT_CNOT
    pl = O.PLACE_AFTER if placement == "after" else O.PLACE_BEFORE
    E0, g0 = O.mcclean_grad(n, axes, angles, t, entangler=ent, placement=pl)
    for mode in ("history", "uncompute"):
        circ = _mcclean(n, L, c, ladder=ladder, placement=placement, grad_mode=mode)
        E, g = circ.grad_run()
        assert abs(E - E0) <= TOL128, (mode, E, E0)
        assert rel_err(g, g0) <= TOL128, (mode, rel_err(g, g0))
    Er = circ.run_expec_val()
    assert abs(Er - O.mcclean_run(n, axes, angles, t, entangler=ent, placement=pl)) <= TOL128


def test_mcclean_many_z_rotations():
    """More Z rotations in a layer than one phase table holds."""
    n, L = 12, 2
    axes = np.full((L, n), 2)
    axes[0, 3] = 0
    rng = np.random.default_rng(11)
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    kind, q0, q1, w = [3, 0, 1], [0, 2, 5], [1, 2, 5], [1.0, 0.6, -0.8]
    c = {"axes": axes, "angles": angles, "kind": np.array(kind), "q0": np.array(q0), "q1": np.array(q1),
         "w": np.array(w)}
    E0, g0 = O.mcclean_grad(n, axes, angles, O.Terms(kind, q0, q1, w))
    for mode in ("history", "uncompute"):
        circ = _mcclean(n, L, c, grad_mode=mode)
        E, g = circ.grad_run()
        assert abs(E - E0) <= TOL128 and rel_err(g, g0) <= TOL128, (mode, rel_err(g, g0))


def test_mcclean_chain_n20_c128_and_c64(golden):
    """The n = 20, L = 50 ZZ-chain golden (reference run, 73 s on one core)."""
    c = golden.case("mcclean", "chain_n20_L50")
    if not c:
        pytest.skip("golden generated without --big")
    for dtype, tol in (("complex128", TOL128), ("complex64", TOL64)):
        circ = _mcclean(20, 50, c, dtype=dtype)
        E, g = circ.grad_run()
        err = rel_err(g, c["grad"])
        print("%s n=20 L=50: |dE| = %.3e, normwise grad error = %.3e" % (dtype, abs(E - float(c["e_grad"])), err))
        assert abs(E - float(c["e_grad"])) <= tol and err <= tol


def test_qaoa_vs_oracle_weighted():
    """Non-integer weights take the real-cost path."""
    from qradient_gb300 import Qaoa

    n, p = 9, 3
    rng = np.random.default_rng(5)
    kind = np.array([3, 3, 3, 2, 2])
    q0 = np.array([0, 1, 2, 4, 7])
    q1 = np.array([3, 5, 8, 4, 7])
    w = np.array([0.7, -1.3, 0.1, 0.45, np.pi / 7])
    betas = rng.uniform(0, np.pi, p)
    gammas = rng.uniform(0, np.pi, p)
    t = O.Terms(kind, q0, q1, w)
    E0, g0 = O.qaoa_grad(n, betas, gammas, t)
    circ = Qaoa(n, obs_dict(n, kind, q0, q1, w), p)
    E, g = circ.grad_run(betas, gammas)
    assert abs(E - E0) <= TOL128 and rel_err(g, g0) <= TOL128


def test_qaoa_regular_vs_oracle():
    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    for n, p, seed in ((16, 3, 1), (18, 2, 2)):
        edges = random_regular_edges(3, n, seed)
        obs = MaxCut(n, edge_set=edges).to_observable()
        rng = np.random.default_rng(seed)
        betas = rng.uniform(0, np.pi, p)
        gammas = rng.uniform(0, np.pi, p)
        t = O.Terms(np.full(len(edges), 3), edges[:, 0], edges[:, 1], np.ones(len(edges)))
        E0, g0 = O.qaoa_grad(n, betas, gammas, t)
        for mode in ("history", "uncompute"):
            circ = Qaoa(n, obs, p, grad_mode=mode)
            E, g = circ.grad_run(betas, gammas)
            assert abs(E - E0) <= TOL128 * max(1, abs(E0)) and rel_err(g, g0) <= TOL128
        tab = circ.classical_ham()
        assert np.array_equal(tab.astype(np.int32), O.maxcut_table(n, edges))


def test_invalid_inputs_raise_value_error():
    from qradient_gb300 import McClean, Qaoa

    zz = np.full((4, 4), None)
    zz[0, 1] = 1.0
    c = McClean(4, {"zz": zz}, 2, axes=np.array([[0, 1, 2, 3], [0, 0, 0, 0]]), angles=np.zeros((2, 4)))
    with pytest.raises(ValueError):
        c.grad_run()
    q = Qaoa(4, {"zz": zz}, 2)
    with pytest.raises(ValueError):
        q.grad_run(np.zeros(3), np.zeros(2))


def test_mcclean_periodic_ladder_vs_oracle():
    """The periodic CNOT ladder (state.py:209-241, periodic=True; its
    permutation is pinned to the reference's own ladder matrices by
    test_oracle_golden.py) through the sweep path, both placements and
    gradient modes, against the oracle; complex64 error stated."""
    from qradient_gb300 import McClean

    for n, L in ((6, 3), (12, 4), (14, 5), (18, 4)):
        rng = np.random.default_rng(n)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        zz = np.full((n, n), None)
        for i in range(n - 1):
            zz[i, i + 1] = 1.0
        x = np.full(n, None)
        x[n // 2] = 0.6
        obs = {"zz": zz, "x": x}
        t = O.Terms.from_dict(n, obs)
        for place in ("before", "after"):
            E0, g0 = O.mcclean_grad(n, axes, angles, t, entangler=O.ENT_CNOT_PERIODIC,
                                    placement=O.PLACE_BEFORE if place == "before" else O.PLACE_AFTER)
            for mode in ("history", "uncompute"):
                c = McClean(n, obs, L, axes=axes, angles=angles, entangler="cnot_periodic", placement=place,
                            grad_mode=mode)
                E, g = c.grad_run()
                assert abs(E - E0) <= TOL128 and rel_err(g, g0) <= TOL128, (n, place, mode, rel_err(g, g0))
                assert abs(c.run_expec_val() - E0) <= TOL128
            c64 = McClean(n, obs, L, axes=axes, angles=angles, entangler="cnot_periodic", placement=place,
                          dtype="complex64")
            E, g = c64.grad_run()
            assert abs(E - E0) <= TOL64 and rel_err(g, g0) <= TOL64, (n, place, rel_err(g, g0))
    with pytest.raises(ValueError):
        McClean(5, {"zz": np.full((5, 5), None)}, 1, entangler="cnot_periodic")


def test_batched_periodic_ladder_vs_oracle():
    """Batched jobs with the periodic ladder: one CTA holds n <= 13
    (complex64); n = 14 runs on the sweep path inside the same graph (the
    ladder's CNOT(n-1, 0) targets the qubit a 2-CTA job splits)."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.batched import Batch

    b = Batch(dtype="complex64")
    jobs = []
    for n, L in ((10, 4), (14, 3), (8, 2)):
        rng = np.random.default_rng(100 + n)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        zz = np.full((n, n), None)
        for i in range(n - 1):
            zz[i, i + 1] = 1.0
        c = McClean(n, {"zz": zz}, L, axes=axes, angles=angles, entangler="cnot_periodic", dtype="complex64")
        jobs.append((b.add(c), n, axes, angles, O.Terms.from_dict(n, {"zz": zz})))
    b.finalize()
    E, grads = b.grad()
    torch.cuda.synchronize()
    for slot, n, axes, angles, t in jobs:
        E0, g0 = O.mcclean_grad(n, axes, angles, t, entangler=O.ENT_CNOT_PERIODIC)
        assert abs(E[slot].item() - E0) <= TOL64, n
        assert rel_err(grads[slot].cpu().numpy().reshape(g0.shape), g0) <= TOL64, n

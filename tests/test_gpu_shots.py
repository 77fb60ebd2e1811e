"""Per-term expectations, projector shots and parameter-shift gradients on the GPU.

* qg_pauli_expectations against the reference's Projector probabilities
  (tests/golden/projectors.npz) at 1e-12 (complex128) / 1e-6 (complex64);
* the exact parameter-shift gradient (sample_grad with shot_num=None)
  against the reference's adjoint gradient goldens at 1e-12: the shifted
  circuits are right;
* projector shots: counts follow Binomial(shots, (1 + <P>) / 2) (chi-square),
  sampled gradients and expectation values scatter around the exact ones
  with the standard deviation the estimator has (z-scores), and a seed
  fixes the draw.  The reference draws with scipy.stats.rv_discrete and
  numpy's Mersenne Twister; these shots use Philox4x32-10, so parity here is
  in distribution, not draw for draw.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, obs_dict, rel_err
from oracle import oracle as O
from oracle import shots as OS

pytestmark = pytest.mark.gpu

SHIFT_CASES = ["pauli_n5_L4", "pauli_n7_L3", "zz01_seed0_n10_L10", "cz_n6_L4", "ini_n6_L3", "zz01_n4_L3"]


def _circuit(golden, name, dtype="complex128", components=False):
    from qradient_gb300 import McClean

    m = next(m for m in golden.cases("mcclean") if m["name"] == name)
    c = golden.case("mcclean", name)
    n, L = m["n"], m["L"]
    circ = McClean(n, obs_dict(n, c["kind"], c["q0"], c["q1"], c["w"]), L, use_observable_components=components,
                   axes=c["axes"].astype(int), angles=c["angles"], dtype=dtype,
                   entangler="cz" if m["ladder"] == "cz" else "cnot")
    return circ, c, m


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-6)])
def test_pauli_expectations_match_reference_projectors(golden, dtype, tol):
    z = np.load(os.path.join(GOLDEN_DIR, "projectors.npz"))
    for name in sorted({k.split("/")[0] for k in z.files}):
        circ, c, m = _circuit(golden, name, dtype)
        circ.state.vec = c["state"]
        e = circ.pauli_expectations().cpu().numpy()
        assert np.max(np.abs(OS.p_plus(e) - z[name + "/p_plus"])) <= tol, name


@pytest.mark.parametrize("name", SHIFT_CASES)
def test_exact_parameter_shift_equals_adjoint_gradient(golden, name):
    circ, c, m = _circuit(golden, name)
    E, g = circ.sample_grad(shot_num=None, ini_state=c.get("ini"))
    assert abs(E - float(c["e_run"])) <= 1e-12 * max(1.0, abs(float(c["e_run"])))
    assert rel_err(g, c["grad"]) <= 1e-12, (name, rel_err(g, c["grad"]))


def test_exact_component_shift_equals_component_gradient():
    """Positive weights (the reference's numpy.random.choice needs them): the
    component-sampling golden circuit of optimizer.npz."""
    from qradient_gb300 import McClean

    z = np.load(os.path.join(GOLDEN_DIR, "optimizer.npz"))
    c = {k.split("/")[-1]: z[k] for k in z.files if k.startswith("comp/comp_n5_L3/")}
    L, n = c["axes"].shape
    seed = 17
    circ = McClean(n, obs_dict(n, c["kind"], c["q0"], c["q1"], c["w"]), L, use_observable_components=True,
                   axes=c["axes"].astype(int), angles=c["angles"])
    np.random.seed(seed)
    E, g = circ.sample_grad_with_component_sampling(shot_num=None)
    np.random.seed(seed)
    p = c["w"] / np.sum(c["w"])
    ks = [int(np.random.choice(np.arange(len(p)), p=p)) for _ in range(L * n)]
    for i in range(L):
        for q in range(n):
            k = ks[i * n + q]
            one = O.Terms(c["kind"][k:k + 1], c["q0"][k:k + 1], c["q1"][k:k + 1], c["w"][k:k + 1])
            _, gk = O.mcclean_grad(n, c["axes"], c["angles"], one)
            assert abs(g[i, q] - gk[i, q]) <= 1e-12 * max(1.0, np.max(np.abs(gk))), (i, q, k)


def test_shot_counts_are_binomial():
    import torch
    from scipy import stats

    from qradient_gb300 import _native

    dev = torch.device("cuda", 0)
    rows, shots = 20000, 50
    ev = torch.tensor([0.3, -0.8, 0.95, 1.0], dtype=torch.float64, device=dev)
    w = torch.tensor([1.0, 2.0, 0.5, 1.5], dtype=torch.float64, device=dev)
    expec = ev.repeat(rows, 1).contiguous()
    est = torch.empty_like(expec)
    total = torch.empty(rows, dtype=torch.float64, device=dev)
    _native.projector_shots(expec, w, shots, seed=12345, offset=7, term_est=est, total=total)
    est = est.cpu().numpy()
    counts = np.rint((est / w.cpu().numpy() + 1.0) * shots / 2).astype(int)
    assert np.allclose(total.cpu().numpy(), est.sum(axis=1), rtol=0, atol=1e-12)
    for k, e in enumerate(ev.cpu().numpy()):
        p = 0.5 * (1 + e)
        if p == 1.0:
            assert np.all(counts[:, k] == shots)
            continue
        obs = np.bincount(counts[:, k], minlength=shots + 1).astype(float)
        exp = stats.binom.pmf(np.arange(shots + 1), shots, p) * rows
        keep = exp >= 5  # pool the tails
        o = np.append(obs[keep], obs[~keep].sum())
        x = np.append(exp[keep], exp[~keep].sum())
        if x[-1] < 5:
            o[-2] += o[-1]
            x[-2] += x[-1]
            o, x = o[:-1], x[:-1]
        chi2 = np.sum((o - x) ** 2 / x)
        pval = stats.chi2.sf(chi2, len(o) - 1)
        assert pval > 1e-4, (k, chi2, pval)
    # the seed and offset select the stream
    est2 = torch.empty((rows, 4), dtype=torch.float64, device=dev)
    _native.projector_shots(expec, w, shots, seed=12345, offset=7, term_est=est2)
    assert np.array_equal(est2.cpu().numpy(), est)
    _native.projector_shots(expec, w, shots, seed=12345, offset=8, term_est=est2)
    assert not np.array_equal(est2.cpu().numpy(), est)


def _shifted_expectations(c, n, L, sign, kind, q0, q1):
    """Oracle <P_k> of every shifted circuit (layer-major, qubit-minor)."""
    out = np.zeros((L * n, len(kind)))
    for i in range(L):
        for q in range(n):
            a = c["angles"].copy()
            a[i, q] += sign * np.pi / 2
            _, st = O.mcclean_run(n, c["axes"], a, O.Terms(c["kind"], c["q0"], c["q1"], c["w"]), want_state=True)
            out[i * n + q] = OS.pauli_expectations(st, n, kind, q0, q1)
    return out


def test_sample_grad_scatter_matches_the_estimator(golden):
    name, shots = "pauli_n5_L4", 4000
    circ, c, m = _circuit(golden, name)
    n, L = m["n"], m["L"]
    _, g_exact = circ.sample_grad(shot_num=None)
    _, g = circ.sample_grad(shot_num=shots, seed=2024)
    _, g_again = circ.sample_grad(shot_num=shots, seed=2024)
    assert np.array_equal(g, g_again)
    ep = _shifted_expectations(c, n, L, +1, c["kind"], c["q0"], c["q1"])
    em = _shifted_expectations(c, n, L, -1, c["kind"], c["q0"], c["q1"])
    sd = np.array([0.5 * np.hypot(OS.estimate_std(ep[r], c["w"], shots), OS.estimate_std(em[r], c["w"], shots))
                   for r in range(L * n)]).reshape(L, n)
    zs = (g - g_exact) / sd
    assert np.max(np.abs(zs)) < 5.0
    # sum of z^2 over L n entries is chi-square with L n degrees of freedom
    from scipy import stats

    chi2 = float(np.sum(zs ** 2))
    assert 1e-4 < stats.chi2.cdf(chi2, zs.size) < 1 - 1e-4, chi2


def test_sample_expec_val_is_unbiased(golden):
    name, shots, reps = "pauli_n7_L3", 200, 400
    circ, c, m = _circuit(golden, name)
    E = circ.run_expec_val()
    e_terms = OS.pauli_expectations(c["state"], m["n"], c["kind"], c["q0"], c["q1"])
    sd = OS.estimate_std(e_terms, c["w"], shots)
    vals = np.array([circ.sample_expec_val(shots, seed=s) for s in range(reps)])
    assert abs(vals.mean() - E) < 5 * sd / np.sqrt(reps)
    assert 0.7 < vals.std() / sd < 1.3
    assert circ.sample_expec_val(shots, seed=3) == circ.sample_expec_val(shots, seed=3)
    k = 2
    vk = np.array([circ.sample_component_expec_val(shots, k, seed=s) for s in range(reps)])
    sdk = OS.estimate_std(e_terms[k:k + 1], c["w"][k:k + 1], shots)
    assert abs(vk.mean() - c["w"][k] * e_terms[k]) < 5 * sdk / np.sqrt(reps)
    # run_expec_val with shots draws from the state it just computed
    np.random.seed(5)
    v = circ.run_expec_val(exact_expec_val=False, shot_num=shots)
    assert abs(v - E) < 6 * sd


def test_batched_term_expectations_and_shift_gradient():
    """The batched kernel's per-term expectations (the projector estimators'
    inputs) against qg_pauli_expectations on the same final states, for a
    single-CTA complex128 job, 2-CTA and 4-CTA complex64 jobs and a 4-CTA
    complex128 job with X, Y, Z and ZZ terms (X and Y on the split qubits); and the parameter-shift gradient through the batched launch
    against the per-circuit path (forced by an explicit |0..0> start)."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.batched import Batch

    for n, L, dtype, tol in ((10, 3, "complex128", 1e-12), (14, 2, "complex64", 2e-5), (14, 2, "complex128", 1e-12),
                             (15, 2, "complex64", 2e-5)):
        rng = np.random.default_rng(n)
        obs = {"zz": np.full((n, n), None), "x": np.full(n, None), "y": np.full(n, None), "z": np.full(n, None)}
        obs["zz"][0, 1] = 0.7
        obs["zz"][2, n - 1] = -0.4
        obs["x"][0] = 0.3      # the top qubit: split across a 2-CTA job
        obs["x"][n - 2] = 0.5
        obs["y"][1] = -0.25
        obs["z"][n // 2] = 0.9
        c = McClean(n, obs, L, axes=rng.integers(0, 3, (L, n)), angles=rng.uniform(0, 2 * np.pi, (L, n)),
                    dtype=dtype)
        b = Batch(dtype=dtype, grad=False, use_graph=False, term_expectations=True)
        P = [rng.uniform(0, 2 * np.pi, (L, n)) for _ in range(3)]
        slots = [b.add(c, params=p) for p in P]
        b.finalize()
        b.execute()
        torch.cuda.synchronize()
        for slot, p in zip(slots, P):
            c.angles = p
            E = c.run_expec_val()
            ref = c.pauli_expectations().cpu().numpy()
            got = b.term_expec[slot].cpu().numpy()
            assert abs(b.expec[slot].item() - E) <= tol * max(1.0, abs(E))
            assert np.max(np.abs(got - ref)) <= tol, (n, got, ref)
        c.angles = P[0]
        E1, g1 = c.sample_grad(shot_num=None)
        e0 = np.zeros(2 ** n, dtype=np.complex128)
        e0[0] = 1.0
        E2, g2 = c.sample_grad(shot_num=None, ini_state=e0)
        assert abs(E1 - E2) <= tol and rel_err(g1, g2) <= tol, (n, rel_err(g1, g2))

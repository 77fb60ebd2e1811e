"""Batched persistent kernel (qg_batch_launch) and the autograd Function.

Every job of a batch must give the same E and gradient as the same circuit
run alone (the per-call sweep path and the CPU oracle): complex128 to 1e-12
normwise, complex64 to 1e-4 against FP64."""
import numpy as np
import pytest

from conftest import obs_dict, rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mc(n, L, seed, ent="cnot", place="before", dtype="complex128", xy=True):
    from qradient_gb300 import McClean

    rng = np.random.default_rng(seed)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    if n >= 3 and xy:
        kind, q0, q1, w = [3, 0, 1, 3], [0, n - 1, 0, 1], [1, n - 1, 0, n - 1], [1.0, 0.3, -0.4, 0.6]
    elif n >= 2:
        kind, q0, q1, w = [3], [0], [1], [1.0]
    else:
        kind, q0, q1, w = [2], [0], [0], [1.0]
    obs = obs_dict(n, np.array(kind), np.array(q0), np.array(q1), np.array(w))
    c = McClean(n, obs, L, axes=axes, angles=angles, entangler=ent, placement=place, dtype=dtype)
    return c, axes, angles, O.Terms(kind, q0, q1, w)


def _oracle(c, axes, angles, t):
    ent = {"cnot": O.ENT_CNOT, "cz": O.ENT_CZ, None: O.ENT_NONE}[c.entangler]
    pl = O.PLACE_AFTER if c.placement == "after" else O.PLACE_BEFORE
    return O.mcclean_grad(c.qnum, axes, angles, t, entangler=ent, placement=pl)


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-4)])
def test_batch_mcclean_matches_oracle(dtype, tol):
    from qradient_gb300.batched import Batch

    specs = [(1, 3, "cnot", "before"), (2, 4, "cz", "after"), (5, 3, "cnot", "after"), (8, 5, "cnot", "before"),
             (10, 2, "cz", "before"), (12, 3, "cnot", "before"), (13, 2, "cnot", "after"), (14, 2, "cz", "before")]
    if dtype == "complex128":
        specs = [s for s in specs if s[0] <= 13]
    b = Batch(dtype=dtype)
    cases = []
    for k, (n, L, ent, pl) in enumerate(specs):
        c, axes, angles, t = _mc(n, L, 100 + k, ent, pl, dtype)
        b.add(c)
        cases.append((c, axes, angles, t))
    E, G = b.grad()
    E = E.cpu().numpy()
    for k, (c, axes, angles, t) in enumerate(cases):
        E0, g0 = _oracle(c, axes, angles, t)
        g = G[k].cpu().numpy().reshape(g0.shape)
        assert abs(E[k] - E0) <= tol, (c.qnum, E[k], E0)
        assert rel_err(g, g0) <= tol, (c.qnum, rel_err(g, g0))


@pytest.mark.parametrize("dtype,tol,n", [("complex128", 1e-12, 14), ("complex64", 1e-4, 15)])
def test_batch_four_cta_clusters_match_oracle(dtype, tol, n):
    """Jobs above the 2-CTA limit run on 4-CTA clusters: the state split by
    its top two qubits, cross-CTA rotations and reductions on both, and the
    CNOT ladder's CNOT(0, 1) a relabelling of the blocks.  Every ladder form,
    X and Y observable terms on both split qubits, QAOA, and a 2-CTA job in
    the same batch, against the oracle."""
    from qradient_gb300 import McClean, Qaoa
    from qradient_gb300.batched import Batch
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    kind, q0, q1 = [3, 0, 1, 0, 1, 3], [0, 1, 0, 0, 1, 1], [1, 1, 0, 0, 1, n - 1]
    w = [1.0, 0.3, -0.4, 0.2, 0.5, 0.6]
    t = O.Terms(kind, q0, q1, w)
    obs = obs_dict(n, np.array(kind), np.array(q0), np.array(q1), np.array(w))
    b = Batch(dtype=dtype)
    cases = []
    for k, (L, ent, pl) in enumerate(((3, "cnot", "before"), (2, "cnot", "after"), (2, "cz", "after"),
                                      (2, "cz", "before"), (2, None, "before"))):
        rng = np.random.default_rng(200 + k)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        c = McClean(n, obs, L, axes=axes, angles=angles, entangler=ent, placement=pl, dtype=dtype)
        b.add(c)
        cases.append(("mc", c, axes, angles))
    c2, axes2, angles2, t2 = _mc(n - 1, 2, 300, dtype=dtype)  # a 2-CTA job beside them
    b.add(c2)
    cases.append(("mc2", c2, axes2, angles2))
    edges = random_regular_edges(3 if n % 2 == 0 else 4, n, 5)
    q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), 2, dtype=dtype)
    rng = np.random.default_rng(5)
    qp = np.stack([rng.uniform(0, np.pi, 2), rng.uniform(0, np.pi, 2)], axis=1)
    b.add(q, params=qp)
    cases.append(("qaoa", q, edges, qp))
    E, G = b.grad()
    assert not b._big and [g[0] for g in b._groups] == [2, 4], [g[0] for g in b._groups]
    E = E.cpu().numpy()
    for k, case in enumerate(cases):
        if case[0] == "qaoa":
            _, qc, ed, prm = case
            tt = O.Terms(np.full(len(ed), 3), ed[:, 0], ed[:, 1], np.ones(len(ed)))
            E0, g0 = O.qaoa_grad(n, prm[:, 0], prm[:, 1], tt)
            g = G[k].cpu().numpy().reshape(-1, 2)
        else:
            _, c, axes, angles = case
            E0, g0 = _oracle(c, axes, angles, t2 if case[0] == "mc2" else t)
            g = G[k].cpu().numpy().reshape(g0.shape)
        assert abs(E[k] - E0) <= tol * max(1.0, abs(E0)), (k, E[k], E0)
        assert rel_err(g, g0) <= tol, (k, rel_err(g, g0))


def test_batch_qaoa_and_mixed_sizes():
    """QAOA and McClean jobs of different sizes in one batch, including a
    circuit too large for shared memory (sweep path inside the same graph)."""
    from qradient_gb300 import Qaoa
    from qradient_gb300.batched import Batch
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    b = Batch(dtype="complex128")
    qcases = []
    for n, p, seed in ((6, 2, 1), (10, 3, 2), (12, 2, 3), (16, 2, 4)):
        edges = random_regular_edges(3, n, seed)
        q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), p)
        rng = np.random.default_rng(seed)
        params = np.stack([rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)], axis=1)
        b.add(q, params=params)
        qcases.append((q, edges, params))
    c, axes, angles, t = _mc(11, 3, 7)
    b.add(c)
    E, G = b.grad()
    for k, (q, edges, params) in enumerate(qcases):
        tt = O.Terms(np.full(len(edges), 3), edges[:, 0], edges[:, 1], np.ones(len(edges)))
        E0, g0 = O.qaoa_grad(q.qnum, params[:, 0], params[:, 1], tt)
        assert abs(float(E[k]) - E0) <= 1e-12 * max(1, abs(E0)), (q.qnum, float(E[k]), E0)
        assert rel_err(G[k].cpu().numpy().reshape(-1, 2), g0) <= 1e-12, q.qnum
    E0, g0 = _oracle(c, axes, angles, t)
    assert abs(float(E[4]) - E0) <= 1e-12 and rel_err(G[4].cpu().numpy().reshape(g0.shape), g0) <= 1e-12


def test_batch_graph_replay_with_new_parameters():
    import torch

    from qradient_gb300.batched import mcclean_batch

    n, L, B = 9, 4, 16
    rng = np.random.default_rng(3)
    axes = rng.integers(0, 3, (L, n))
    zz = np.full((n, n), None)
    zz[0, 1] = 1.0
    b = mcclean_batch(n, L, axes, {"zz": zz}, B, dtype="complex128")
    t = O.Terms([3], [0], [1], [1.0])
    for rep in range(2):
        P = rng.uniform(0, 2 * np.pi, (B, L * n))
        b.params_flat.copy_(torch.as_tensor(P.reshape(-1)))
        E, G = b.grad()
        for k in (0, B // 2, B - 1):
            E0, g0 = O.mcclean_grad(n, axes, P[k].reshape(L, n), t)
            assert abs(float(E[k]) - E0) <= 1e-12
            assert rel_err(G[k].cpu().numpy().reshape(L, n), g0) <= 1e-12


def test_batch_equals_single_call():
    """A job gives the same numbers in a batch as the same circuit alone."""
    from qradient_gb300.batched import Batch

    c, axes, angles, t = _mc(12, 6, 21, dtype="complex128")
    E1, g1 = c.grad_run()
    b = Batch(dtype="complex128")
    for _ in range(5):
        b.add(c)
    E, G = b.grad()
    for k in range(5):
        assert abs(float(E[k]) - E1) <= 1e-12
        assert rel_err(G[k].cpu().numpy().reshape(g1.shape), g1) <= 1e-12


def test_autograd_matches_finite_differences_and_oracle():
    import torch

    from qradient_gb300.autograd import mcclean_expectation, qaoa_expectation
    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    c, axes, angles, t = _mc(7, 3, 5)
    a = torch.tensor(angles, dtype=torch.float64, device="cuda", requires_grad=True)
    E = mcclean_expectation(a, c)
    E.backward()
    E0, g0 = _oracle(c, axes, angles, t)
    assert abs(E.item() - E0) <= 1e-12
    assert rel_err(a.grad.cpu().numpy(), g0) <= 1e-12
    h = 1e-5
    fd = np.zeros_like(g0)
    for i in range(angles.shape[0]):
        for q in range(angles.shape[1]):
            p = angles.copy()
            p[i, q] += h
            c.angles = p
            ep = c.run_expec_val()
            p[i, q] -= 2 * h
            c.angles = p
            em = c.run_expec_val()
            fd[i, q] = (ep - em) / (2 * h)
    c.angles = angles
    assert np.max(np.abs(fd - g0)) < 1e-8
    # QAOA through autograd
    edges = random_regular_edges(3, 8, 2)
    q = Qaoa(8, MaxCut(8, edge_set=edges).to_observable(), 2)
    prm = torch.tensor([[0.3, 0.7], [1.1, 0.2]], dtype=torch.float64, device="cuda", requires_grad=True)
    Eq = qaoa_expectation(prm, q)
    Eq.backward()
    tt = O.Terms(np.full(len(edges), 3), edges[:, 0], edges[:, 1], np.ones(len(edges)))
    Eq0, gq0 = O.qaoa_grad(8, [0.3, 1.1], [0.7, 0.2], tt)
    assert abs(Eq.item() - Eq0) <= 1e-12 and rel_err(prm.grad.cpu().numpy(), gq0) <= 1e-12


def test_batched_autograd_n14_complex64_vs_fd():
    """Config-3 shape (n=14, L=30, shared axes) at a reduced batch: complex64
    batched gradients against central differences of complex128 runs
    (h = 1e-5) and against the FP64 oracle."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.autograd import batched_expectation
    from qradient_gb300.batched import mcclean_batch

    n, L, B = 14, 30, 8
    rng = np.random.default_rng(14)
    axes = rng.integers(0, 3, (L, n))
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    b = mcclean_batch(n, L, axes, {"zz": zz}, B, dtype="complex64")
    P = torch.tensor(rng.uniform(0, 2 * np.pi, (B, L * n)), dtype=torch.float64, device="cuda", requires_grad=True)
    E = batched_expectation(P, b)
    E.sum().backward()
    t = O.Terms(np.full(n - 1, 3), np.arange(n - 1), np.arange(1, n), np.ones(n - 1))
    ref = McClean(n, {"zz": zz}, L, axes=axes, angles=np.zeros((L, n)), dtype="complex128")
    worst = 0.0
    for k in (0, B - 1):
        Pk = P[k].detach().cpu().numpy().reshape(L, n)
        E0, g0 = O.mcclean_grad(n, axes, Pk, t)
        gk = P.grad[k].cpu().numpy().reshape(L, n)
        worst = max(worst, rel_err(gk, g0))
        assert abs(E[k].item() - E0) <= 1e-4
        # central differences on a few entries
        for (i, q) in ((0, 0), (L // 2, n // 2), (L - 1, n - 1)):
            h = 1e-5
            p = Pk.copy()
            p[i, q] += h
            ref.angles = p
            ep = ref.run_expec_val()
            p[i, q] -= 2 * h
            ref.angles = p
            em = ref.run_expec_val()
            assert abs((ep - em) / (2 * h) - g0[i, q]) < 1e-7
            assert abs(gk[i, q] - g0[i, q]) <= 1e-4 * max(1.0, np.max(np.abs(g0)))
    print("batched complex64 n=14 L=30: normwise gradient error vs FP64 oracle %.2e" % worst)
    assert worst <= 1e-4


def test_config3_full_batch_and_complex128_check():
    """Config 3 as stated: 4096 parameter vectors (uniform [0, 2 pi)) of a
    McClean n=14 L=30 circuit with shared random axes in one CUDA-graph
    replay, complex64 with FP32 sums, every job's E and gradient written;
    sampled jobs against the FP64 oracle (the reference's grad_run
    restated, mc_clean.py:47-78) and against central differences (h =
    1e-5) of complex128 runs; and the complex128 check: n=14 complex128 jobs
    exceed the 2-CTA limit (13) and run on 4-CTA clusters of the same
    kernel, in one graph replay, checked against the oracle to 1e-12."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.batched import mcclean_batch

    n, L, B = 14, 30, 4096
    rng = np.random.default_rng(3)
    axes = rng.integers(0, 3, (L, n))
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    t = O.Terms(np.full(n - 1, 3), np.arange(n - 1), np.arange(1, n), np.ones(n - 1))
    P = rng.uniform(0, 2 * np.pi, (B, L * n))
    b = mcclean_batch(n, L, axes, {"zz": zz}, B, dtype="complex64")
    b.params_flat.copy_(torch.as_tensor(P.reshape(-1), device=b.params_flat.device))
    E, _ = b.grad()
    E, _ = b.grad()  # the graph replay
    torch.cuda.synchronize()
    Eh = E.cpu().numpy()
    G = b.grads_flat.cpu().numpy().reshape(B, L, n)
    assert np.all(np.isfinite(Eh)) and np.all(np.isfinite(G))
    ref = McClean(n, {"zz": zz}, L, axes=axes, angles=np.zeros((L, n)), dtype="complex128")
    worst = 0.0
    for k in rng.choice(B, 6, replace=False):
        E0, g0 = O.mcclean_grad(n, axes, P[k].reshape(L, n), t)
        worst = max(worst, rel_err(G[k], g0))
        assert abs(Eh[k] - E0) <= 1e-4, k
        for (i, q) in ((0, 0), (L - 1, n - 1)):
            h = 1e-5
            a = P[k].reshape(L, n).copy()
            a[i, q] += h
            ref.angles = a
            ep = ref.run_expec_val()
            a[i, q] -= 2 * h
            ref.angles = a
            em = ref.run_expec_val()
            assert abs((ep - em) / (2 * h) - g0[i, q]) < 1e-8
            assert abs(G[k, i, q] - g0[i, q]) <= 1e-4 * max(1.0, np.max(np.abs(g0)))
    print("config 3, 4096 vectors, complex64: worst normwise gradient error of 6 sampled jobs vs FP64 %.2e" % worst)
    assert worst <= 1e-4
    # the complex128 check (4-CTA clusters)
    B2 = 32
    b2 = mcclean_batch(n, L, axes, {"zz": zz}, B2, dtype="complex128")
    assert not b2._big and [g[0] for g in b2._groups] == [4]
    b2.params_flat.copy_(torch.as_tensor(P[:B2].reshape(-1), device=b2.params_flat.device))
    b2.grad()
    E2, _ = b2.grad()
    torch.cuda.synchronize()
    G2 = b2.grads_flat.cpu().numpy().reshape(B2, L, n)
    for k in (0, B2 - 1):
        E0, g0 = O.mcclean_grad(n, axes, P[k].reshape(L, n), t)
        assert abs(E2[k].item() - E0) <= 1e-12 and rel_err(G2[k], g0) <= 1e-12, (k, rel_err(G2[k], g0))


def test_batch_launch_marks_jobs_it_cannot_hold():
    """qg_batch_launch sizes shared memory by max_qubits; a job above it is
    not run (the kernel checks each job) and gets NaN outputs, the others
    run as usual."""
    import math

    import torch

    from qradient_gb300 import _lib, _native
    from qradient_gb300.batched import Batch

    b = Batch(dtype="complex64", use_graph=False)
    (c1, ax1, an1, t1), (c2, _, _, _) = _mc(8, 2, 1, dtype="complex64"), _mc(10, 2, 2, dtype="complex64")
    b.add(c1)
    b.add(c2)
    b.finalize()
    assert [g[0] for g in b._groups] == [1]
    cl, jobs, nj, maxq, ws = b._groups[0]
    lib = _lib.load()
    _lib.check(lib.qg_batch_launch(_lib.QG_C64, _native.ptr(jobs), nj, 8, cl, _native.ptr(ws), ws.numel(),
                                   _native.stream_handle(b.device)))
    torch.cuda.synchronize()
    E = b.expec.cpu().numpy()
    E0, g0 = _oracle(c1, ax1, an1, t1)
    assert abs(E[0] - E0) <= 1e-4 and math.isnan(E[1])
    G = b.grads_flat.cpu().numpy()
    assert rel_err(G[: g0.size].reshape(g0.shape), g0) <= 1e-4
    assert np.all(np.isnan(G[g0.size: g0.size + 20]))

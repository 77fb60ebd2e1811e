"""Continuous-batching server: every request's result equals the same
request served alone, across mixed sizes, kinds and dtypes; admission keeps
the in-flight footprint within the budget."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _mix(seed, count):
    from qradient_gb300 import McClean, Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        dtype = "complex128" if rng.random() < 0.5 else "complex64"
        if rng.random() < 0.6:
            n = int(rng.integers(4, 17))
            L = int(rng.integers(1, 6))
            zz = np.full((n, n), None)
            for i in range(n - 1):
                zz[i, i + 1] = 1.0
            c = McClean(n, {"zz": zz}, L, axes=rng.integers(0, 3, (L, n)), angles=np.zeros((L, n)), dtype=dtype)
            p = rng.uniform(0, 2 * np.pi, (L, n))
        else:
            n = int(rng.integers(3, 9)) * 2
            p_ = int(rng.integers(1, 4))
            c = Qaoa(n, MaxCut(n, edge_set=random_regular_edges(3, n, k)).to_observable(), p_, dtype=dtype)
            p = np.stack([rng.uniform(0, np.pi, p_), rng.uniform(0, np.pi, p_)], axis=1)
        op = "grad" if rng.random() < 0.8 else "run"
        out.append((c, p, op, dtype))
    return out


def _alone(c, p, op):
    from qradient_gb300 import McClean

    if isinstance(c, McClean):
        c.angles = p
        return c.grad_run() if op == "grad" else (c.run_expec_val(), None)
    return c.grad_run(p[:, 0], p[:, 1]) if op == "grad" else (c.run_expec_val(p[:, 0], p[:, 1]), None)


def test_results_equal_alone_and_in_the_mix():
    from qradient_gb300.serving import Server, latency_stats

    reqs = _mix(5, 40)
    srv = Server(hbm_budget=2 << 30, streams=3, max_batch=16)
    sched = [(0.002 * i, c, p, op, dt) for i, (c, p, op, dt) in enumerate(reqs)]
    done = srv.serve(sched)
    assert len(done) == len(reqs)
    by_id = {r.rid: r for r in done}
    for i, (c, p, op, dt) in enumerate(reqs):
        r = by_id[i]
        E, g = _alone(c, p, op)
        tol = 1e-12 if dt == "complex128" else 1e-5
        assert abs(r.expec - E) <= tol * max(1.0, abs(E)), (i, r.expec, E)
        if op == "grad":
            assert rel_err(r.grad, g) <= tol, (i, rel_err(r.grad, g))
    st = latency_stats(done)
    assert st["p99_ms"] >= st["p50_ms"] > 0
    assert srv.in_use == 0


def test_admission_respects_the_budget():
    from qradient_gb300 import McClean
    from qradient_gb300.serving import Server

    n, L = 18, 2
    zz = np.full((n, n), None)
    zz[0, 1] = 1.0
    circs = [McClean(n, {"zz": zz}, L, axes=np.zeros((L, n), dtype=int), angles=np.zeros((L, n))) for _ in range(4)]
    srv = Server(hbm_budget=None, streams=4)
    one = circs[0].native().workspace_bytes(0, 2)
    srv.budget = int(one * 1.5) + 65536       # room for one large request at a time
    for c in circs:
        srv.submit(c, np.full((L, n), 0.3), "grad", "complex128")
    peak = 0
    while srv.queue or srv.inflight:
        srv.step()
        peak = max(peak, srv.in_use)
        assert srv.in_use <= srv.budget
    assert len(srv.finished) == 4 and peak > 0
    with pytest.raises(MemoryError):
        srv.submit(McClean(24, {"zz": np.full((24, 24), None)}, 1, axes=np.zeros((1, 24), dtype=int),
                           angles=np.zeros((1, 24))), np.zeros((1, 24)), "grad", "complex128")

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


def _chain(n, L, seed, dtype):
    from qradient_gb300 import McClean

    rng = np.random.default_rng(seed)
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    c = McClean(n, {"zz": zz}, L, axes=rng.integers(0, 3, (L, n)), angles=np.zeros((L, n)), dtype=dtype)
    return c, rng.uniform(0, 2 * np.pi, (L, n))


def test_large_requests_alone_equal_in_the_mix():
    """The serving population's sizes (McClean up to n=24 with L up to 60,
    QAOA up to n=24): requests beyond the shared-memory kernel run on the
    sweep path on their own streams, overlapping each other and the batched
    small requests; each result equals the request served alone."""
    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges
    from qradient_gb300.serving import Server

    reqs = []
    for k, (n, L, dt) in enumerate([(24, 60, "complex128"), (22, 40, "complex64"), (20, 60, "complex128"),
                                    (17, 25, "complex64"), (12, 30, "complex128"), (10, 5, "complex64")]):
        c, p = _chain(n, L, 100 + k, dt)
        reqs.append((c, p, "grad" if k != 3 else "run", dt))
    for k, (n, p_, dt) in enumerate([(24, 6, "complex128"), (18, 3, "complex64"), (12, 2, "complex128")]):
        q = Qaoa(n, MaxCut(n, edge_set=random_regular_edges(3, n, 7 + k)).to_observable(), p_, dtype=dt)
        rng = np.random.default_rng(k)
        reqs.append((q, np.stack([rng.uniform(0, np.pi, p_), rng.uniform(0, np.pi, p_)], 1), "grad", dt))
    srv = Server(streams=4)
    done = srv.serve([(0.001 * i, c, p, op, dt) for i, (c, p, op, dt) in enumerate(reqs)])
    assert len(done) == len(reqs) and not srv.failed
    by_id = {r.rid: r for r in done}
    for i, (c, p, op, dt) in enumerate(reqs):
        E, g = _alone(c, p, op)
        tol = 1e-12 if dt == "complex128" else 1e-5
        r = by_id[i]
        assert abs(r.expec - E) <= tol * max(1.0, abs(E)), (i, r.expec, E)
        if op == "grad":
            assert rel_err(r.grad, g) <= tol, (i, rel_err(r.grad, g))
        if c._native is not None:
            c._native.release_workspaces()
    assert srv.in_use == 0


def test_malformed_and_cancelled_requests():
    """Host-side failures: wrong parameter counts and non-finite parameters
    are refused at submission (ValueError); a queued request can be
    cancelled; the others complete and the budget returns to zero."""
    from qradient_gb300.serving import Server

    srv = Server(streams=2)
    c, p = _chain(8, 3, 1, "complex128")
    with pytest.raises(ValueError):
        srv.submit(c, p[:2], "grad")
    bad = p.copy()
    bad[1, 2] = np.nan
    with pytest.raises(ValueError):
        srv.submit(c, bad, "grad")
    with pytest.raises(ValueError):
        srv.submit(c, p, "gradient")
    r0 = srv.submit(c, p, "grad")
    r1 = srv.submit(c, p, "run")
    r2 = srv.submit(c, p, "grad")
    assert srv.cancel(r1.rid) is True
    done = srv.drain()
    assert sorted(r.rid for r in done) == [r0.rid, r2.rid]
    assert [r.rid for r in srv.failed] == [r1.rid] and r1.error == "cancelled"
    assert srv.cancel(r0.rid) is False
    assert srv.in_use == 0
    E, g = _alone(c, p, "grad")
    assert abs(r2.expec - E) <= 1e-12 and rel_err(r2.grad, g) <= 1e-12
    # refused entries of a served schedule are recorded, the rest served
    done = Server(streams=2).serve([(0.0, c, p, "grad", "complex128"), (0.0, c, p[:1], "grad", "complex128")])
    assert len(done) == 1


def test_launch_and_allocation_failures_are_contained(monkeypatch):
    """A batched launch that raises fails only its own requests; a
    workspace allocation that raises (out of device memory) fails only its
    request; both give their footprint and stream back, and the same server
    then serves new requests correctly.  The failures are raised on the
    host; no GPU work faults."""
    import torch

    from qradient_gb300 import _native, batched
    from qradient_gb300.serving import Server

    srv = Server(streams=2)
    small, ps = _chain(9, 4, 3, "complex128")
    large, pl = _chain(18, 3, 4, "complex128")
    orig_exec = batched.Batch.execute
    orig_ws = _native.NativeCircuit.workspace

    def failing_exec(self):
        raise RuntimeError("injected launch failure")

    def failing_ws(self, dtype, op, device):
        raise torch.cuda.OutOfMemoryError("injected allocation failure")

    monkeypatch.setattr(batched.Batch, "execute", failing_exec)
    monkeypatch.setattr(_native.NativeCircuit, "workspace", failing_ws)
    a = srv.submit(small, ps, "grad")
    b = srv.submit(large, pl, "grad")
    srv.drain()
    assert a.failed and "injected launch failure" in a.error
    assert b.failed and "injected allocation failure" in b.error
    assert srv.in_use == 0 and all(s is None for s in srv.stream_busy) and not srv.inflight
    monkeypatch.setattr(batched.Batch, "execute", orig_exec)
    monkeypatch.setattr(_native.NativeCircuit, "workspace", orig_ws)
    c = srv.submit(small, ps, "grad")
    d = srv.submit(large, pl, "grad")
    srv.drain()
    assert c.done and not c.failed and d.done and not d.failed
    for r, (circ, p) in ((c, (small, ps)), (d, (large, pl))):
        E, g = _alone(circ, p, "grad")
        assert abs(r.expec - E) <= 1e-12 and rel_err(r.grad, g) <= 1e-12
    assert srv.in_use == 0

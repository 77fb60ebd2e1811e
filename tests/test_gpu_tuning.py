"""The autotuner's knobs keep results exact, and the tuner picks and caches.

Every fusion depth (tile bits) and grid shape the tuner may choose must give
the reference's gradient (goldens, 1e-12 in complex128, 1e-5 in complex64),
and so must batches whose jobs are split over 2-CTA clusters from a smaller
qubit count than the default."""
import json

import numpy as np
import pytest

from conftest import obs_dict, rel_err
from test_gpu_batched import _mc, _oracle

pytestmark = pytest.mark.gpu

CASES = ["chain_n12_L20", "chain_n14_L30", "chain_n16_L50", "zz01_seed0_n10_L10", "pauli_n9_L2"]


def _golden_circuit(golden, name, dtype):
    from qradient_gb300 import McClean

    m = next(m for m in golden.cases("mcclean") if m["name"] == name)
    c = golden.case("mcclean", name)
    circ = McClean(m["n"], obs_dict(m["n"], c["kind"], c["q0"], c["q1"], c["w"]), m["L"],
                   axes=c["axes"].astype(int), angles=c["angles"], dtype=dtype,
                   entangler="cz" if m["ladder"] == "cz" else "cnot")
    return circ, c


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-5)])
def test_every_candidate_matches_reference(golden, dtype, tol):
    from qradient_gb300 import tuning

    for name in CASES:
        circ, c = _golden_circuit(golden, name, dtype)
        for mode in ("history", "uncompute"):
            circ.grad_mode = mode
            extra = [(9, 2, 1), (6, 0, 1), (6, 0, 2)] + ([(13, 0, 1)] if dtype == "complex64" else [(5, 0, 1)])
            for t, ctas, f in tuning.sweep_candidates(circ._dtype_code, circ.qnum) + extra:
                circ.set_tuning(t, ctas, f)
                E, g = circ.grad_run()
                assert abs(E - float(c["e_grad"])) <= tol * max(1.0, abs(float(c["e_grad"]))), (name, t, ctas, f)
                assert rel_err(g, c["grad"]) <= tol, (name, mode, t, ctas, f, rel_err(g, c["grad"]))
                assert abs(circ.run_expec_val() - float(c["e_run"])) <= tol * max(1.0, abs(float(c["e_run"])))


def test_qaoa_candidates_match_reference(golden):
    from qradient_gb300 import Qaoa, tuning

    for name in ("reg3_n14_p2", "edges10_n12_p10"):
        c = golden.case("qaoa", name)
        n = int(max(c["q1"].max(), c["q0"].max())) + 1
        q = Qaoa(n, obs_dict(n, c["kind"], c["q0"], c["q1"], c["w"]), c["betas"].size)
        for t, ctas, f in tuning.sweep_candidates(q._dtype_code, n):
            q.set_tuning(t, ctas, f)
            E, g = q.grad_run(c["betas"], c["gammas"])
            assert rel_err(g, c["grad"]) <= 1e-12, (name, t, ctas, f)


def test_tuner_picks_applies_and_caches(golden, tmp_path, monkeypatch):
    from qradient_gb300 import tuning

    monkeypatch.setenv("QG_TUNING_CACHE", str(tmp_path / "tune.json"))
    circ, c = _golden_circuit(golden, "chain_n16_L50", "complex128")
    r = tuning.tune_circuit(circ, op="grad", reps=2)
    assert (r["tile_bits"], r["ctas_per_sm"], r["flags"]) in tuning.sweep_candidates(circ._dtype_code, 16)
    assert len(r["timings"]) == len(tuning.sweep_candidates(circ._dtype_code, 16))
    assert all(t["ms"] > 0 for t in r["timings"])
    t_eff, _, f_eff = tuning.get_tuning(circ.native(), circ._dtype_code)
    if r["tile_bits"] == 0:
        # the default plan: the same effective values as an untuned circuit
        fresh, _ = _golden_circuit(golden, "chain_n16_L50", "complex128")
        assert (t_eff, f_eff) == tuple(tuning.get_tuning(fresh.native(), fresh._dtype_code)[::2])
    else:
        assert t_eff == min(r["tile_bits"], 16) and f_eff == r["flags"]
    data = json.load(open(tmp_path / "tune.json"))
    assert len(data) == 1
    # a second circuit of the same shape takes the cached choice without timing
    circ2, _ = _golden_circuit(golden, "chain_n16_L50", "complex128")
    r2 = tuning.tune_circuit(circ2, op="grad")
    assert r2 == json.loads(json.dumps(r))
    E, g = circ2.grad_run()
    assert rel_err(g, c["grad"]) <= 1e-12
    # the autotune flag does the same on first use
    from qradient_gb300 import McClean

    circ3 = McClean(16, circ.observable.info, 50, axes=c["axes"].astype(int), angles=c["angles"], autotune=True)
    E3, g3 = circ3.grad_run()
    assert rel_err(g3, c["grad"]) <= 1e-12


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-4)])
def test_batch_cluster_split_matches_oracle(dtype, tol):
    from qradient_gb300.batched import SINGLE_MAX, Batch

    single = SINGLE_MAX[1 if dtype == "complex64" else 0]
    specs = [(single - 2, 3, "cnot", "before"), (single - 1, 2, "cz", "after"), (single, 3, "cnot", "after"),
             (5, 2, "cnot", "before")]
    cases = []
    for k, (n, L, ent, pl) in enumerate(specs):
        cases.append(_mc(n, L, 300 + k, ent, pl, dtype))
    for cluster_from in (single + 1, single, single - 2):
        b = Batch(dtype=dtype, cluster_from=cluster_from)
        for c, axes, angles, t in cases:
            b.add(c)
        E, G = b.grad()
        E = E.cpu().numpy()
        for k, (c, axes, angles, t) in enumerate(cases):
            E0, g0 = _oracle(c, axes, angles, t)
            assert abs(E[k] - E0) <= tol, (cluster_from, c.qnum)
            assert rel_err(G[k].cpu().numpy().reshape(g0.shape), g0) <= tol, (cluster_from, c.qnum)


def test_tune_batch_keeps_results(tmp_path, monkeypatch):
    import torch

    from qradient_gb300 import tuning
    from qradient_gb300.batched import Batch

    monkeypatch.setenv("QG_TUNING_CACHE", str(tmp_path / "tune.json"))
    b = Batch(dtype="complex64")
    cases = []
    for k in range(64):
        c, axes, angles, t = _mc(12, 6, 500 + (k % 4), dtype="complex64")
        b.add(c)
        cases.append((c, axes, angles, t))
    b.finalize()
    E0, _ = b.grad()
    E0 = E0.clone()
    r = tuning.tune_batch(b, reps=2)
    assert r["cluster_from"] in [t["cluster_from"] for t in r["timings"]]
    E1, G1 = b.grad()
    assert torch.allclose(E1, E0, rtol=0, atol=1e-5)
    c, axes, angles, t = cases[0]
    Eo, go = _oracle(c, axes, angles, t)
    assert rel_err(G1[0].cpu().numpy().reshape(go.shape), go) <= 1e-4

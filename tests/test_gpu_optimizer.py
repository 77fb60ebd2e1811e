"""Device optimiser steps, training loops and component sampling on the GPU.

Against tests/golden/optimizer.npz (the reference's own optimization.py and
grad_run_with_component_sampling, tests/golden/make_golden.py --optimizer):

* the update kernels (qg_adam_step, qg_gd_step, qg_plateau_step) fed the
  golden gradients reproduce the reference's parameters bit for bit;
* the device gradient at each golden step's parameters matches the
  reference's to 1e-12 (complex128);
* McCleanOpt / QaoaOpt run free on the device and follow the reference's
  histories to the tolerance the optimiser allows (free_run_tolerance);
* a training step returns nothing to the host (CUDA sync debug mode);
* the max_iter bookkeeping raises where the reference's does.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, rel_err
from test_optimizer_oracle import (RULES, RUN_SEEDS, RUNS, draw_components, free_run_tolerance, gd_decay, hyper,
                                   zz_chain)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def opt_golden():
    z = np.load(os.path.join(GOLDEN_DIR, "optimizer.npz"))

    def case(pre):
        return {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}

    return case


def _obs(n, c):
    from conftest import obs_dict

    return obs_dict(n, c["kind"], c["q0"], c["q1"], c["w"])


@pytest.mark.parametrize("name", sorted(RULES))
def test_device_update_rules_bit_exact(opt_golden, name):
    import torch

    from qradient_gb300 import optimization as opt_mod

    c = opt_golden("rule/%s/" % name)
    kind, h = RULES[name]
    dev = torch.device("cuda", 0)
    opt = getattr(opt_mod, kind)(torch.as_tensor(c["p0"], device=dev), hyper(name, h))
    grads = torch.as_tensor(c["grads"], device=dev)
    costs = torch.as_tensor(c["costs"], device=dev)
    row = torch.empty_like(opt.parameters)
    for k in range(len(c["grads"])):
        opt.step(grads[k], costs[k:k + 1], history_row=row)
        p = opt.parameters.cpu().numpy()
        assert np.array_equal(p, c["hist"][k + 1]), (name, k, np.max(np.abs(p - c["hist"][k + 1])))
        assert np.array_equal(row.cpu().numpy(), p)
        assert opt.step_size == c["rates"][k]


def _make(name, c, dtype="complex128"):
    from qradient_gb300 import McClean, Qaoa

    kind, h, comp = RUNS[name]
    if name.startswith("qaoa"):
        n = int(np.max(c["edges"])) + 1
        return Qaoa(n, _obs(n, c), c["betas"].size, dtype=dtype)
    L, n = c["axes"].shape
    return McClean(n, _obs(n, c), L, use_observable_components=comp, axes=c["axes"].astype(int),
                   angles=c["angles"].copy(), dtype=dtype)


@pytest.mark.parametrize("name", sorted(RUNS))
def test_device_gradient_at_each_golden_step(opt_golden, name):
    import torch

    c = opt_golden("run/%s/" % name)
    kind, h, comp = RUNS[name]
    hist, costs, grads = c["param_history"], c["cost_history"], c["grads"]
    steps = len(costs) - 1
    circ = _make(name, c)
    ks = draw_components(c["w"], RUN_SEEDS.get(name, 0), steps) if comp else [None] * steps
    dev = torch.device("cuda", 0)
    for it in range(steps):
        p = torch.as_tensor(hist[it], device=dev)
        nat = circ.native()
        e, g = nat.grad(p, circ._dtype_code, dev, circ._grad_op(nat), component=ks[it])
        assert abs(e.item() - costs[it]) <= 1e-12 * max(1.0, abs(costs[it])), (name, it)
        assert rel_err(g.cpu().numpy(), grads[it].reshape(-1)) <= 1e-12, (name, it)


def _run_opt(name, c, circ, steps):
    from qradient_gb300.optimization import McCleanOpt, QaoaOpt

    kind, h, comp = RUNS[name]
    spec = dict(hyper(name, h), name=kind)
    if name.startswith("qaoa"):
        o = QaoaOpt(circ, spec, c["betas"], c["gammas"], max_iter=steps + 1)
        for _ in range(steps):
            o.step()
    else:
        o = McCleanOpt(circ, spec, max_iter=steps + 1)
        np.random.seed(RUN_SEEDS.get(name, 0))
        for _ in range(steps):
            o.step(component_sampling=comp)
    return o


@pytest.mark.parametrize("name", sorted(RUNS))
def test_device_training_run_follows_reference(opt_golden, name):
    c = opt_golden("run/%s/" % name)
    kind, h, comp = RUNS[name]
    hist, costs = c["param_history"], c["cost_history"]
    steps = len(costs) - 1
    o = _run_opt(name, c, _make(name, c), steps)
    tol = free_run_tolerance(kind)
    assert np.array_equal(o.param_history[0], hist[0])
    assert np.max(np.abs(o.param_history - hist)) <= tol, name
    assert np.max(np.abs(o.cost_history - costs)) <= tol * max(1.0, np.max(np.abs(costs))), name
    assert o.iter == steps
    if not name.startswith("qaoa"):
        assert np.array_equal(o.circuit.angles.cpu().numpy(), o.param_history[steps])


def test_complex64_training_run_stays_close(opt_golden):
    """complex64 gradients (~1e-6 relative) through the same Adam loop."""
    name = "qaoa_adam_n8_p3"
    c = opt_golden("run/%s/" % name)
    steps = len(c["cost_history"]) - 1
    o = _run_opt(name, c, _make(name, c, dtype="complex64"), steps)
    assert np.max(np.abs(o.param_history - c["param_history"])) <= 1e-4
    assert np.max(np.abs(o.cost_history - c["cost_history"])) <= 1e-4


@pytest.mark.parametrize("name,n,seed", [("comp_n5_L3", 5, 51), ("comp_n7_L4", 7, 52)])
@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-5)])
def test_component_sampling_matches_reference(opt_golden, name, n, seed, dtype, tol):
    from qradient_gb300 import McClean

    c = opt_golden("comp/%s/" % name)
    L = c["axes"].shape[0]
    circ = McClean(n, _obs(n, c), L, use_observable_components=True, axes=c["axes"].astype(int),
                   angles=c["angles"], dtype=dtype)
    np.random.seed(seed)
    for d in range(len(c["e"])):
        e, g = circ.grad_run_with_component_sampling()
        assert abs(e - c["e"][d]) <= tol * max(1.0, abs(c["e"][d])), (name, d)
        assert rel_err(g, c["grads"][d]) <= tol, (name, d)


def test_training_step_stays_on_device():
    """After the first step (which sizes the workspace), steps never
    synchronise the host with the GPU: torch's sync debug mode turns any
    device-to-host copy or stream synchronisation into an error."""
    import torch

    from qradient_gb300 import McClean, Qaoa
    from qradient_gb300.optimization import McCleanOpt, QaoaOpt
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    n, L = 12, 6
    rng = np.random.default_rng(3)
    mc = McClean(n, {"zz": zz_chain(n)}, L, axes=rng.integers(0, 3, (L, n)), angles=rng.uniform(0, 6, (L, n)))
    q = Qaoa(10, MaxCut(10, edge_set=random_regular_edges(3, 10, 2)).to_observable(), 3)
    opts = [McCleanOpt(mc, {"name": "Adam", "step_size": 0.01}, max_iter=20),
            McCleanOpt(mc, {"name": "RateDecayOnPlateau", "step_size": 0.01}, max_iter=20),
            McCleanOpt(mc, {"name": "GradientDescent", "step_size": 0.01, "decay_function": gd_decay}, max_iter=20),
            QaoaOpt(q, {"name": "Adam", "step_size": 0.01}, np.full(3, 0.3), np.full(3, 0.2), max_iter=20)]
    for o in opts:
        o.step()
    torch.cuda.synchronize()
    torch.cuda.set_sync_debug_mode("error")
    try:
        for o in opts:
            for _ in range(4):
                o.step()
    finally:
        torch.cuda.set_sync_debug_mode("default")
    torch.cuda.synchronize()
    for o in opts:
        assert o.iter == 5
        assert np.all(np.isfinite(o.param_history[:6]))
        assert np.all(o.cost_history[:5] != 0)


def test_max_iter_bookkeeping_matches_reference():
    """optimization.py:70-91 with max_iter = 3: two steps fill the history,
    the third updates the parameters and then fails writing param_history[3],
    a fourth fails writing cost_history[3]."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.optimization import McCleanOpt

    n, L = 6, 2
    rng = np.random.default_rng(9)
    mc = McClean(n, {"zz": zz_chain(n)}, L, axes=rng.integers(0, 3, (L, n)), angles=rng.uniform(0, 6, (L, n)))
    o = McCleanOpt(mc, {"name": "Adam", "step_size": 0.1}, max_iter=3)
    o.step()
    o.step()
    before = o.optimizer.parameters.clone()
    with pytest.raises(IndexError):
        o.step()
    assert o.iter == 3
    assert not torch.equal(before, o.optimizer.parameters)
    with pytest.raises(IndexError):
        o.step()
    o.reset()
    assert o.iter == 0
    assert np.array_equal(o.param_history[0], o.optimizer.parameters.cpu().numpy())

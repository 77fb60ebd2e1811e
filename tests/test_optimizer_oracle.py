"""Optimiser updates and component sampling: the oracle against the reference.

tests/golden/optimizer.npz holds what the reference's own optimiser classes
(qradient/optimization.py) and McClean.grad_run_with_component_sampling
(mc_clean.py:80-115) produced (tests/golden/make_golden.py --optimizer).  The
oracle's update rules must reproduce the rule cases bit for bit, and the
oracle's gradient + update loop the training runs; the GPU tests then use the
same goldens for the device path.  The last tests cover the host logic of the
training loops that needs no GPU."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, rel_err
from oracle import optimization as OO
from oracle import oracle as O

RULES = {
    "adam_default": ("Adam", {}),
    "adam_custom": ("Adam", {"step_size": 0.05, "beta1": 0.8, "beta2": 0.99, "eps": 1e-6}),
    "gd_plain": ("GradientDescent", {"step_size": 0.1}),
    "gd_decay": ("GradientDescent", {"step_size": 0.2}),
    "plateau": ("RateDecayOnPlateau", {"step_size": 0.3, "plateau_length": 3, "decay_rate": 0.5}),
}

RUNS = {
    # name: (optimizer name, hyper-parameters, component sampling)
    "mcclean_adam_n6_L4": ("Adam", {"step_size": 0.05}, False),
    "mcclean_gd_n5_L3": ("GradientDescent", {"step_size": 0.1}, False),
    "mcclean_plateau_n6_L3": ("RateDecayOnPlateau", {"step_size": 0.9, "plateau_length": 2, "decay_rate": 0.5},
                              False),
    "qaoa_adam_n8_p3": ("Adam", {"step_size": 0.05}, False),
    "mcclean_adam_comp_n6_L3": ("Adam", {"step_size": 0.05}, True),
}
RUN_SEEDS = {"mcclean_adam_comp_n6_L3": 45}


def gd_decay(step_size, it):
    """The decay function the golden GradientDescent cases used."""
    return step_size / (1.0 + 0.25 * it)


def zz_chain(n):
    """Observable 'zz' array with Z_i Z_{i+1} for i < n - 1."""
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    return zz


def hyper(name, base):
    h = dict(base)
    if name in ("gd_decay", "mcclean_gd_n5_L3"):
        h["decay_function"] = gd_decay
    return h


@pytest.fixture(scope="module")
def opt_golden():
    z = np.load(os.path.join(GOLDEN_DIR, "optimizer.npz"))

    def case(pre):
        return {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}

    return case


def oracle_optimizer(kind, p0, h):
    cls = {"Adam": OO.Adam, "GradientDescent": OO.GradientDescent, "RateDecayOnPlateau": OO.RateDecayOnPlateau}[kind]
    return cls(p0, **h)


@pytest.mark.parametrize("name", sorted(RULES))
def test_update_rules_bit_exact(opt_golden, name):
    c = opt_golden("rule/%s/" % name)
    kind, h = RULES[name]
    opt = oracle_optimizer(kind, c["p0"], hyper(name, h))
    for k in range(len(c["grads"])):
        opt.step(c["grads"][k], c["costs"][k])
        assert np.array_equal(opt.parameters, c["hist"][k + 1]), (name, k)
        assert opt.step_size == c["rates"][k]


def component_terms(c, k):
    return O.Terms(c["kind"][k:k + 1], c["q0"][k:k + 1], c["q1"][k:k + 1], c["w"][k:k + 1])


def draw_components(w, seed, draws):
    """The draws of mc_clean.py:102 after numpy.random.seed(seed)."""
    np.random.seed(seed)
    p = np.asarray(w) / np.sum(w)
    return [int(np.random.choice(np.arange(len(w)), p=p)) for _ in range(draws)]


@pytest.mark.parametrize("name,n,seed", [("comp_n5_L3", 5, 51), ("comp_n7_L4", 7, 52)])
def test_component_sampling_semantics(opt_golden, name, n, seed):
    """The reference's sampled gradient is the gradient of w_k P_k for the
    drawn term k, with E the full expectation value."""
    c = opt_golden("comp/%s/" % name)
    full = O.Terms(c["kind"], c["q0"], c["q1"], c["w"])
    ks = draw_components(c["w"], seed, len(c["e"]))
    E_full, _ = O.mcclean_grad(n, c["axes"], c["angles"], full)
    for d, k in enumerate(ks):
        _, g = O.mcclean_grad(n, c["axes"], c["angles"], component_terms(c, k))
        assert abs(c["e"][d] - E_full) <= 1e-12
        assert rel_err(g, c["grads"][d]) <= 1e-12, (name, d, k)


def run_grad(name, c, params, comp_k=None):
    """Oracle (E, grad) of a training-run case at the given parameters."""
    terms = O.Terms(c["kind"], c["q0"], c["q1"], c["w"])
    p = np.asarray(params)
    if name.startswith("qaoa"):
        n = int(np.max(c["edges"])) + 1
        return O.qaoa_grad(n, p[:, 0], p[:, 1], terms)
    n = p.shape[1]
    E, g = O.mcclean_grad(n, c["axes"], p, terms)
    if comp_k is not None:
        _, g = O.mcclean_grad(n, c["axes"], p, component_terms(c, comp_k))
    return E, g


def free_run_tolerance(kind):
    """Adam divides each gradient by sqrt(v_hat) + 1e-8.  Gradients that are
    zero up to rounding (rotations outside the observable's light cone) are
    ~1e-17 noise in any implementation, and Adam turns a 1e-17 difference
    into a parameter difference of up to step_size * 1e-9, which then feeds
    every later gradient; free-running Adam trajectories therefore agree to
    about 1e-9, not to rounding.  The other rules multiply the gradient by
    the step size and stay at rounding level."""
    return 1e-7 if kind == "Adam" else 1e-10


@pytest.mark.parametrize("name", sorted(RUNS))
def test_training_run_steps(opt_golden, name):
    """Each step of a McCleanOpt / QaoaOpt run: the oracle's E and gradient at
    the golden parameters match the reference's to 1e-12, and the oracle's
    update fed the reference's gradients reproduces the parameter history bit
    for bit."""
    c = opt_golden("run/%s/" % name)
    kind, h, comp = RUNS[name]
    hist, costs, grads = c["param_history"], c["cost_history"], c["grads"]
    steps = len(costs) - 1
    ks = draw_components(c["w"], RUN_SEEDS.get(name, 0), steps) if comp else [None] * steps
    opt = oracle_optimizer(kind, hist[0], hyper(name, h))
    for it in range(steps):
        E, g = run_grad(name, c, hist[it], ks[it])
        assert abs(E - costs[it]) <= 1e-12 * max(1.0, abs(costs[it])), (name, it)
        assert rel_err(g, grads[it]) <= 1e-12, (name, it)
        opt.step(grads[it], costs[it])
        assert np.array_equal(opt.parameters, hist[it + 1]), (name, it)


@pytest.mark.parametrize("name", sorted(RUNS))
def test_training_runs_free(opt_golden, name):
    """Oracle gradient + oracle update over a whole run, starting from the
    golden initial parameters only."""
    c = opt_golden("run/%s/" % name)
    kind, h, comp = RUNS[name]
    hist, costs = c["param_history"], c["cost_history"]
    steps = len(costs) - 1
    tol = free_run_tolerance(kind)
    ks = draw_components(c["w"], RUN_SEEDS.get(name, 0), steps) if comp else [None] * steps
    opt = oracle_optimizer(kind, hist[0], hyper(name, h))
    for it in range(steps):
        E, g = run_grad(name, c, opt.parameters, ks[it])
        assert abs(E - costs[it]) <= tol * max(1.0, abs(costs[it])), (name, it)
        opt.step(g, E)
        assert np.max(np.abs(opt.parameters - hist[it + 1])) <= tol, (name, it)


def test_unknown_optimizer_raises_before_any_device_work():
    from qradient_gb300 import McClean
    from qradient_gb300.optimization import McCleanOpt

    zz = np.full((3, 3), None)
    zz[0, 1] = 1.0
    c = McClean(3, {"zz": zz}, 2, axes=np.zeros((2, 3), dtype=int), angles=np.zeros((2, 3)))
    with pytest.raises(ValueError, match="No optimizer"):
        McCleanOpt(c, {"name": "Nesterov"})
    with pytest.raises(ValueError, match="No optimizer"):
        McCleanOpt(c, "Adam")


def test_no_cpu_fallback():
    import torch

    if torch.cuda.is_available():
        pytest.skip("checks the CPU-only behaviour")
    from qradient_gb300 import McClean
    from qradient_gb300.optimization import Adam, McCleanOpt

    zz = np.full((3, 3), None)
    zz[0, 1] = 1.0
    c = McClean(3, {"zz": zz}, 2, axes=np.zeros((2, 3), dtype=int), angles=np.zeros((2, 3)))
    with pytest.raises(RuntimeError, match="CUDA"):
        McCleanOpt(c, {"name": "Adam"})
    with pytest.raises(RuntimeError, match="CUDA"):
        Adam(np.zeros(4), {})

"""Parity at the configured sizes: every gradient entry of the GPU path
against the CPU oracle (oracle/qg_oracle.c, the reference's grad_run
restated and pinned to the reference's own outputs up to n = 20 by
test_oracle_golden.py).

- McClean n=24 L=50 complex128, the benchmarked circuit (same seeded axes
  and angles as bench.py), in both gradient modes; the complex64 per-entry
  error against the same FP64 oracle is printed and bounded.
- The same circuit with the CZ ladder after the rotations.
- n=20 L=100, n=28 L=4 and n=30 L=2 (complex128 and complex64 where it fits).
- QAOA MaxCut on seeded 3-regular graphs: n=20 p=10, n=24 p=10, n=26 p=4,
  with the integer cost table bit-exact at each n.

Tolerances: complex128 normwise ||g - g_ref||_inf / ||g_ref||_inf <= 1e-12
and |E - E_ref| <= 1e-12 (mc_clean.py:47-78, qaoa.py:40-70); complex64
normwise <= 1e-4.  The oracle keeps the reference's state history where it
fits in host memory and otherwise uncomputes psi (validated against the
history mode on the CPU)."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 1e-4

_cache = {}


def _mem_available():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_AVPHYS_PAGES")


def _oracle_uncompute(n, states_history):
    """History mode where its states fit in half the free host memory, else
    uncompute (three states); skip when even that does not fit."""
    S = (2 ** n) * 16
    avail = _mem_available()
    if (states_history + 2) * S <= 0.5 * avail:
        return False
    if 4 * S <= 0.8 * avail:
        return True
    pytest.skip("host memory %.1f GiB is too small for the n=%d oracle" % (avail / 2 ** 30, n))


def _chain_inputs(n, L, seed):
    """bench.py's workload: numpy default_rng(seed), axes then angles."""
    rng = np.random.default_rng(seed)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    return axes, angles, {"zz": zz}


def _chain_terms(n):
    return O.Terms(np.full(n - 1, O.ZZ), np.arange(n - 1), np.arange(1, n), np.ones(n - 1))


def _oracle_mcclean(n, L, seed, ent, place):
    key = ("mc", n, L, seed, ent, place)
    if key not in _cache:
        axes, angles, _ = _chain_inputs(n, L, seed)
        unc = _oracle_uncompute(n, L + 1)
        e = {"cnot": O.ENT_CNOT, "cz": O.ENT_CZ}[ent]
        p = {"before": O.PLACE_BEFORE, "after": O.PLACE_AFTER}[place]
        _cache[key] = O.mcclean_grad(n, axes, angles, _chain_terms(n), entangler=e, placement=p, uncompute=unc)
    return _cache[key]


def _gpu_mcclean(n, L, seed, dtype="complex128", mode="auto", ent="cnot", place="before"):
    from qradient_gb300 import McClean

    axes, angles, obs = _chain_inputs(n, L, seed)
    c = McClean(n, obs, L, axes=axes, angles=angles, dtype=dtype, grad_mode=mode, entangler=ent, placement=place)
    E, g = c.grad_run()
    if c._native is not None:
        c._native.release_workspaces()
    return E, g


def _entry_stats(g, g_ref):
    """Per-entry errors: absolute, and relative to the largest |g_ref| entry."""
    d = np.abs(np.asarray(g) - np.asarray(g_ref)).ravel()
    scale = max(np.max(np.abs(g_ref)), 1e-300)
    return {"max": float(d.max()), "p99": float(np.percentile(d, 99)), "median": float(np.median(d)),
            "normwise": float(d.max() / scale)}


def _check128(name, E, g, E0, g0):
    st = _entry_stats(g, g0)
    print("%s complex128 vs oracle: |dE| %.2e, per entry max %.2e p99 %.2e median %.2e, normwise %.2e" %
          (name, abs(E - E0), st["max"], st["p99"], st["median"], st["normwise"]))
    assert abs(E - E0) <= TOL128, (name, E, E0)
    assert st["normwise"] <= TOL128, (name, st)


def _check64(name, E, g, E0, g0):
    st = _entry_stats(g, g0)
    print("%s complex64 vs FP64 oracle: |dE| %.2e, per entry max %.2e p99 %.2e median %.2e, normwise %.2e "
          "(%d entries)" % (name, abs(E - E0), st["max"], st["p99"], st["median"], st["normwise"], np.size(g0)))
    assert abs(E - E0) <= TOL64 and st["normwise"] <= TOL64, (name, st)


@pytest.mark.parametrize("mode", ["history", "uncompute"])
def test_mcclean_n24_L50_c128_every_entry(mode):
    """The benchmarked circuit: 1200 gradient entries and E against the oracle."""
    E0, g0 = _oracle_mcclean(24, 50, 24, "cnot", "before")
    E, g = _gpu_mcclean(24, 50, 24, mode=mode)
    _check128("McClean n=24 L=50 (%s)" % mode, E, g, E0, g0)


def test_mcclean_n24_L50_c64_error_per_entry():
    E0, g0 = _oracle_mcclean(24, 50, 24, "cnot", "before")
    E, g = _gpu_mcclean(24, 50, 24, dtype="complex64")
    _check64("McClean n=24 L=50", E, g, E0, g0)


def test_mcclean_n24_L50_cz_after():
    """The layer as BASELINE's configuration text words it: rotations, then
    the CZ ladder on neighbours."""
    E0, g0 = _oracle_mcclean(24, 50, 24, "cz", "after")
    E, g = _gpu_mcclean(24, 50, 24, ent="cz", place="after")
    _check128("McClean n=24 L=50 CZ after", E, g, E0, g0)
    E, g = _gpu_mcclean(24, 50, 24, dtype="complex64", ent="cz", place="after")
    _check64("McClean n=24 L=50 CZ after", E, g, E0, g0)


def test_mcclean_n20_L100():
    E0, g0 = _oracle_mcclean(20, 100, 20, "cnot", "before")
    for mode in ("history", "uncompute"):
        E, g = _gpu_mcclean(20, 100, 20, mode=mode)
        _check128("McClean n=20 L=100 (%s)" % mode, E, g, E0, g0)
    E, g = _gpu_mcclean(20, 100, 20, dtype="complex64")
    _check64("McClean n=20 L=100", E, g, E0, g0)


@pytest.mark.parametrize("n,L", [(28, 4), (30, 2)])
def test_mcclean_largest_every_entry(n, L):
    E0, g0 = _oracle_mcclean(n, L, n, "cnot", "before")
    E, g = _gpu_mcclean(n, L, n, mode="uncompute")
    _check128("McClean n=%d L=%d (uncompute)" % (n, L), E, g, E0, g0)
    E, g = _gpu_mcclean(n, L, n, dtype="complex64", mode="uncompute")
    _check64("McClean n=%d L=%d (uncompute)" % (n, L), E, g, E0, g0)


def _fd(c, i, q, h=1e-5):
    a = np.array(c.angles, copy=True)
    p = a.copy()
    p[i, q] += h
    c.angles = p
    ep = c.run_expec_val()
    p[i, q] -= 2 * h
    c.angles = p
    em = c.run_expec_val()
    c.angles = a
    return (ep - em) / (2 * h)


def test_n24_L50_forward_and_finite_differences():
    """Independent of the oracle: forward E equals grad_run's E, and central
    differences (h = 1e-5) of run_expec_val agree with three entries."""
    from qradient_gb300 import McClean

    axes, angles, obs = _chain_inputs(24, 50, 24)
    c = McClean(24, obs, 50, axes=axes, angles=angles)
    E, g = c.grad_run()
    assert abs(c.run_expec_val() - E) <= 1e-12
    for (i, q) in ((0, 0), (25, 11), (49, 23)):
        assert abs(_fd(c, i, q) - g[i, q]) <= 1e-8, (i, q)
    c._native.release_workspaces()


@pytest.mark.parametrize("n,p", [(20, 10), (24, 10), (26, 4)])
def test_qaoa_config_sizes(n, p):
    """QAOA MaxCut on a seeded random 3-regular graph, beta and gamma
    uniform in [0, pi): E and the 2p gradient entries against the oracle,
    the integer cost table bit-exact, and 100 Philox shots from the final
    state drawn from its support."""
    import torch

    from qradient_gb300 import Qaoa
    from qradient_gb300.circuit_logic.qaoa import maxcut_table
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    edges = random_regular_edges(3, n, n)
    rng = np.random.default_rng(n)
    betas, gammas = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    t = O.Terms(np.full(len(edges), O.ZZ), edges[:, 0], edges[:, 1], np.ones(len(edges)))
    table = maxcut_table(n, edges).cpu().numpy()
    assert np.array_equal(table, O.maxcut_table(n, edges)), "cost table differs"
    del table
    E0, g0 = O.qaoa_grad(n, betas, gammas, t, uncompute=_oracle_uncompute(n, 2 * p + 1))
    for mode in ("history", "uncompute"):
        q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), p, grad_mode=mode)
        E, g = q.grad_run(betas, gammas)
        _check128("QAOA n=%d p=%d (%s)" % (n, p, mode), E, g, E0, g0)
        q._native.release_workspaces()
    q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), p)
    assert abs(q.run_expec_val(betas, gammas) - E0) <= TOL128
    shots = q.sample(100, seed=n).cpu().numpy()
    assert shots.shape == (100,) and shots.min() >= 0 and shots.max() < 2 ** n
    prob = np.abs(q.state.tensor[torch.as_tensor(shots, device=q.state.tensor.device)].cpu().numpy()) ** 2
    assert np.all(prob > 0)
    q._native.release_workspaces()

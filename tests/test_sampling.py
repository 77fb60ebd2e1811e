"""Shot sampling (Qaoa.sample / qg_sample): Philox4x32-10 stream and
inverse-CDF draws from |psi|^2.

CPU part: a plain restatement of Philox4x32-10 (Salmon et al., SC'11)
against the published known-answer vectors.  GPU part: a chi-square test of
the sampled histogram against |psi|^2 (the reference's rv_discrete draws use
another RNG, so distributions, not draws, are compared), and the draws
against the CPU restatement of the same stream."""
import numpy as np
import pytest

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85


def philox4x32_10(ctr, key):
    c = list(ctr)
    k0, k1 = key
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF,
             p0 & 0xFFFFFFFF]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c


def test_philox_known_answers():
    assert philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _u01(a, b):
    return (((a >> 5) << 26) | (b >> 6)) / 9007199254740992.0


@pytest.mark.gpu
def test_samples_follow_born_rule():
    from scipy import stats

    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    n, p = 8, 2
    q = Qaoa(n, MaxCut(n, edge_set=random_regular_edges(3, n, 3)).to_observable(), p)
    q.run_expec_val(np.array([0.4, 1.1]), np.array([0.9, 0.3]))
    prob = np.abs(q.state.vec) ** 2
    shots = q.sample(200000, seed=1234).cpu().numpy()
    assert shots.min() >= 0 and shots.max() < 2 ** n
    counts = np.bincount(shots, minlength=2 ** n)
    keep = prob * shots.size > 5
    f_exp = prob[keep] / prob[keep].sum() * counts[keep].sum()
    chi = stats.chisquare(counts[keep], f_exp)
    assert chi.pvalue > 1e-4, chi
    # the 100-shot estimate of the QAOA cost, as in the configs
    few = q.sample(100, seed=7).cpu().numpy()
    est = q.classical_ham()[few].mean()
    exact = q.run_expec_val(np.array([0.4, 1.1]), np.array([0.9, 0.3]))
    assert abs(est - exact) < 6 * np.sqrt(np.var(q.classical_ham(), ddof=0) / 100 + 1e-12) + 1e-9


@pytest.mark.gpu
def test_draws_reproduce_the_philox_stream():
    import torch

    from qradient_gb300.circuit_logic.qaoa import sample_state

    n = 6
    rng = np.random.default_rng(2)
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    v /= np.linalg.norm(v)
    t = torch.as_tensor(v, device="cuda")
    seed, offset, k = 0x1234567890ABCDEF, 17, 512
    got = sample_state(t, k, seed=seed, offset=offset).cpu().numpy()
    cdf = np.cumsum(np.abs(v) ** 2)
    want = []
    for s in range(k):
        ctr = s + offset
        c = philox4x32_10([ctr & 0xFFFFFFFF, ctr >> 32, 0, 0], [seed & 0xFFFFFFFF, seed >> 32])
        u = _u01(c[0], c[1]) * cdf[-1]
        want.append(int(np.searchsorted(cdf, u, side="right")))
    same = np.mean(np.array(want) == got)
    assert same >= 0.99, same

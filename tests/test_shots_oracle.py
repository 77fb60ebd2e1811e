"""Projector shots: the oracle against the reference's Projector class, and
the host-side argument checks (no GPU needed).

tests/golden/projectors.npz holds ||Pi_+ psi||^2 for every observable term
on the golden final states, computed with the reference's own Projector
(observable.py:126-177; tests/golden/make_golden.py --projectors).  The
oracle's p = (1 + <P>) / 2 must match it; the GPU tests then check the
device expectations against the same numbers."""
import os
import warnings

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from oracle import shots as OS


@pytest.fixture(scope="module")
def projectors():
    return np.load(os.path.join(GOLDEN_DIR, "projectors.npz"))


def test_oracle_projector_probabilities_match_reference(golden, projectors):
    names = sorted({k.split("/")[0] for k in projectors.files})
    assert len(names) >= 10
    for name in names:
        c = golden.case("mcclean", name)
        vec = c["state"]
        n = int(np.log2(vec.size))
        e = OS.pauli_expectations(vec, n, c["kind"], c["q0"], c["q1"])
        assert np.max(np.abs(OS.p_plus(e) - projectors[name + "/p_plus"])) <= 1e-12, name
        assert abs(np.dot(e, c["w"]) - float(c["e_run"])) <= 1e-12, name


def test_shot_arguments_are_checked_before_device_work():
    from qradient_gb300 import McClean

    zz = np.full((3, 3), None)
    zz[0, 1] = 1.0
    c = McClean(3, {"zz": zz}, 1, axes=np.zeros((1, 3), dtype=int), angles=np.zeros((1, 3)))
    for bad in (0, -3, 2.5):
        with pytest.raises(ValueError, match="shot_num"):
            c.sample_expec_val(bad)
        with pytest.raises(ValueError, match="shot_num"):
            c.sample_grad(shot_num=bad)


def test_qaoa_sample_grad_is_a_stub_as_in_the_reference():
    """qaoa.py:72-81 only warns; so does the counterpart here."""
    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut

    q = Qaoa(4, MaxCut(4, edge_set=[(0, 1), (1, 2), (2, 3)]).to_observable(), 2)
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        assert q.sample_grad([0.1, 0.2], [0.3, 0.4]) is None
    assert any("Not implemented" in str(r.message) for r in rec)

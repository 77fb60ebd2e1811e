"""Pauli-sum observable, parsed from the reference's dictionary format.

Mirrors ``qradient/physical_components/observable.py``: keys 'x', 'y', 'z'
hold length-n weight arrays (None = absent) and 'zz' a strict upper-triangular
n x n array (observable.py:12-17).  Validation raises and warns as there
(shape check :19-26, lower triangle :57-64, unknown keys :106-117, near-zero
weights :119-124).  The matrix is never formed for the device path; the
device applies the terms directly.  ``matrix`` builds the reference's sparse
matrix on demand for small systems.
"""
import warnings

import numpy as np

from .. import _lib

KNOWN_KEYS = ("x", "y", "z", "zz")


def _weight_check(weight, component):
    if abs(weight) < 1e-15:
        warnings.warn("Weight in observable {} is zero or almost zero. If you don't want to include it, "
                      "set it to None.".format(component))


class Observable:
    def __init__(self, qubit_number, observable, store_components=False):
        if not isinstance(observable, dict):
            raise ValueError("observable must be a dict with keys among %s" % (KNOWN_KEYS,))
        self.qnum = qubit_number
        self.info = observable
        self.store_components = store_components
        for key, v in observable.items():
            if v is None:
                continue
            for s in np.shape(v):
                if s != qubit_number:
                    raise ValueError("Inconsistent shapes in observable dictionary. Cannot infer qubit_number.")
        for key in observable:
            if key not in KNOWN_KEYS:
                warnings.warn("Unknown element of observable {} will be ignored.".format(key))
        kind, q0, q1, w = [], [], [], []
        n = qubit_number
        for key, k in (("x", _lib.QG_PAULI_X), ("y", _lib.QG_PAULI_Y), ("z", _lib.QG_PAULI_Z)):
            arr = observable.get(key)
            if arr is None:
                continue
            for q, v in enumerate(arr):
                if v is not None:
                    _weight_check(v, key)
                    kind.append(k), q0.append(q), q1.append(q), w.append(float(v))
        zz = observable.get("zz")
        if zz is not None:
            zz = np.asarray(zz, dtype=object)
            for i in range(n):
                for j in range(i + 1):
                    if zz[i, j] is not None:
                        raise ValueError("zz of observable should be a upper triangular {} by {} matrix. Diagonal "
                                         "and lower triangle should contain None's, not {}.".format(n, n, zz[i, j]))
                for j in range(i + 1, n):
                    if zz[i, j] is not None:
                        _weight_check(zz[i, j], "zz")
                        kind.append(_lib.QG_PAULI_ZZ), q0.append(i), q1.append(j), w.append(float(zz[i, j]))
        self.terms = (np.array(kind, np.int32), np.array(q0, np.int32), np.array(q1, np.int32),
                      np.array(w, np.float64))
        self.num_components = len(w)
        if store_components and self.num_components:
            ws = np.array(w)
            self.weight_distribution = ws / ws.sum()
        self._matrix = None

    @property
    def matrix(self):
        """The reference's sparse matrix sum_k w_k P_k (observable.py:34-73)."""
        if self._matrix is None:
            import scipy.sparse as sp

            n = self.qnum
            ops = {
                0: sp.csr_matrix(np.array([[0, 1], [1, 0]], dtype=complex)),
                1: sp.csr_matrix(np.array([[0, -1j], [1j, 0]], dtype=complex)),
                2: sp.csr_matrix(np.array([[1, 0], [0, -1]], dtype=complex)),
            }
            eye = lambda k: sp.identity(2 ** k, dtype=complex, format="csr")
            m = sp.csr_matrix((2 ** n, 2 ** n), dtype=complex)
            for k, a, b, wt in zip(*self.terms):
                if k == _lib.QG_PAULI_ZZ:
                    op = sp.kron(sp.kron(sp.kron(sp.kron(eye(a), ops[2]), eye(b - a - 1)), ops[2]), eye(n - b - 1))
                else:
                    op = sp.kron(sp.kron(eye(a), ops[int(k)]), eye(n - a - 1))
                m = m + wt * op
            self._matrix = m.asformat("csr")
        return self._matrix

    def diagonal_terms(self):
        """(kind, q0, q1, w) restricted to Z and ZZ terms."""
        kind, q0, q1, w = self.terms
        sel = kind >= _lib.QG_PAULI_Z
        return kind[sel], q0[sel], q1[sel], w[sel]

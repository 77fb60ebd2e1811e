"""Stand-in for the missing ``qradient.physical_components`` API.

Test infrastructure only: ``make_golden.py`` registers this module as
``qradient.physical_components`` so that the reference's *unmodified*
``qradient/circuit_logic/{base,mc_clean,qaoa}.py`` can run and produce the
golden vectors committed under ``tests/golden/``.  The checked-out reference
does not import on its own: ``circuit_logic/mc_clean.py:2`` and ``qaoa.py:2``
import a ``Gates`` class that ``physical_components/__init__.py:1-2`` does not
export, and the circuit code calls ``State``/``Observable`` methods that the
snapshot does not define.

Every operator below restates the mathematics of the reference's
``physical_components`` (citations per method) with sparse matrices built from
Kronecker products, so that the arithmetic the circuit code performs is the
reference's own (CSR mat-vec, numpy elementwise, ``vdot``-style sums).

Qubit ``q`` is the most significant of the ``n`` index bits (bit ``n-1-q``),
as in ``kron(id(2^q), op, id(2^(n-q-1)))`` (``state.py:84-88``).
"""
import warnings

import numpy as np
import scipy.sparse as sp

_X = sp.csr_matrix(np.array([[0.0, 1.0], [1.0, 0.0]], dtype=complex))
_Y = sp.csr_matrix(np.array([[0.0, -1.0j], [1.0j, 0.0]], dtype=complex))
_Z = sp.csr_matrix(np.array([[1.0, 0.0], [0.0, -1.0]], dtype=complex))
_P0 = sp.csr_matrix(np.array([[1.0, 0.0], [0.0, 0.0]], dtype=complex))
_P1 = sp.csr_matrix(np.array([[0.0, 0.0], [0.0, 1.0]], dtype=complex))


def _eye(k):
    return sp.identity(2 ** k, dtype=complex, format="csr")


def _embed(n, q, op):
    """op acting on qubit q of n: id(2^q) (x) op (x) id(2^(n-q-1))."""
    return sp.kron(sp.kron(_eye(q), op, format="csr"), _eye(n - q - 1), format="csr")


def _embed2(n, q0, op0, q1, op1):
    """op0 on qubit q0 and op1 on qubit q1 (q0 < q1)."""
    m = sp.kron(_eye(q0), op0, format="csr")
    m = sp.kron(m, _eye(q1 - q0 - 1), format="csr")
    m = sp.kron(m, op1, format="csr")
    return sp.kron(m, _eye(n - q1 - 1), format="csr")


def _cnot(n, c, t):
    """CNOT with control c and target t (c < t), ``state.py:336-345``."""
    return (_embed(n, c, _P0) + _embed2(n, c, _P1, t, _X)).asformat("csr")


def _cz(n, a, b):
    """CZ on qubits a < b: |0><0|_a (x) 1 + |1><1|_a (x) Z_b."""
    return (_embed(n, a, _P0) + _embed2(n, a, _P1, b, _Z)).asformat("csr")


class Gates:
    """Holder of precomputed operators, the API used at ``mc_clean.py:16-20``
    and ``qaoa.py:11-14`` (``Gates`` itself is missing from the snapshot)."""

    def __init__(self, qnum):
        self.qnum = qnum

    def add_xrots(self):
        # state.py:81-88: xrot[i] = -i X_i
        self.xrot = [-1.0j * _embed(self.qnum, q, _X) for q in range(self.qnum)]
        return self

    def add_yrots(self):
        # state.py:133-140: yrot[i] = -i Y_i
        self.yrot = [-1.0j * _embed(self.qnum, q, _Y) for q in range(self.qnum)]
        return self

    def add_zrots(self):
        # state.py:159-166: 0/1 masks of bit(n-1-q) == 0 / == 1
        n = self.qnum
        idx = np.arange(2 ** n)
        self.zrot_pos = np.zeros((n, 2 ** n), dtype=complex)
        self.zrot_neg = np.zeros((n, 2 ** n), dtype=complex)
        for q in range(n):
            bit = (idx >> (n - 1 - q)) & 1
            self.zrot_pos[q] = (bit == 0)
            self.zrot_neg[q] = (bit == 1)
        return self

    def add_cnot_ladder(self, periodic=False):
        # state.py:209-241: ladder[0] = (prod even-pair CNOTs) . (prod odd-pair CNOTs)
        # as a matrix product, ladder[1] its inverse.
        n = self.qnum
        upper = n if periodic else n - 1
        even = [_cnot(n, i, (i + 1) % n) for i in range(0, upper, 2)]
        odd = [_cnot(n, i, (i + 1) % n) for i in range(1, upper, 2)]
        l0 = _eye(n)
        l1 = _eye(n)
        for m in even:
            l0 = l0.dot(m)
        for m in odd:
            l0 = l0.dot(m)
            l1 = l1.dot(m)
        for m in even:
            l1 = l1.dot(m)
        self.cnot_ladder = [l0.asformat("csr"), l1.asformat("csr")]
        return self

    def use_cz_ladder(self):
        """Replace the CNOT ladder with a CZ ladder on neighbours (q, q+1).

        Not part of the reference: used to produce goldens for the CZ
        entangler placed where the reference places its ladder."""
        n = self.qnum
        m = _eye(n)
        for q in range(n - 1):
            m = m.dot(_cz(n, q, q + 1))
        self.cnot_ladder = [m.asformat("csr"), m.asformat("csr")]
        return self

    def add_x_summed(self):
        # state.py:107-119: 1/2 sum_q (-i X_q)
        n = self.qnum
        m = sp.csr_matrix((2 ** n, 2 ** n), dtype=complex)
        for q in range(n):
            m = m + 0.5 * (-1.0j * _embed(n, q, _X))
        self.x_summed = m.asformat("csr")
        return self

    def add_classical_ham(self, observable, include_individual_components=False):
        # state.py:261-297: diagonal of the z / zz part of the observable
        n = self.qnum
        info = observable.info
        zvec = np.array([1.0, -1.0])
        ones = lambda k: np.full(2 ** k, 1.0)
        self.classical_ham = np.zeros(2 ** n, dtype="double")
        comps = []
        if "z" in info and info["z"] is not None:
            for q, w in enumerate(info["z"]):
                if w is not None:
                    c = w * np.kron(ones(q), np.kron(zvec, ones(n - q - 1)))
                    self.classical_ham += c
                    comps.append(c)
        if "zz" in info:
            for i in range(n):
                for j in range(i + 1, n):
                    w = info["zz"][i, j]
                    if w is not None:
                        c = w * np.kron(ones(i), np.kron(zvec, np.kron(ones(j - i - 1), np.kron(zvec, ones(n - j - 1)))))
                        self.classical_ham += c
                        comps.append(c)
        if include_individual_components:
            self.classical_ham_components = np.array(comps)
        return self


class State:
    """Statevector with the gate methods the circuit code calls
    (``mc_clean.py:36-77``, ``qaoa.py:33-69``)."""

    def __init__(self, qubit_number, ini="0"):
        self.qnum = qubit_number
        self._ini = ini
        self.reset()

    def reset(self, ini=None):
        # state.py:61-71; the circuit code passes '+' once (qaoa.py:17) and
        # expects later reset() calls to remember it.
        if ini is not None:
            self._ini = ini
        n = self.qnum
        if self._ini == "0":
            self.vec = np.zeros(2 ** n, dtype=complex)
            self.vec[0] = 1.0
        elif self._ini == "+":
            self.vec = 2.0 ** (-0.5 * n) * np.ones(2 ** n, dtype=complex)
        else:
            raise ValueError("Invalid initialization format {}.".format(self._ini))

    # state.py:90-97
    def xrot(self, angle, i):
        self.vec = np.sin(0.5 * angle) * self.gates.xrot[i].dot(self.vec) + np.cos(0.5 * angle) * self.vec

    def dxrot(self, angle, i):
        self.vec = 0.5 * np.cos(0.5 * angle) * self.gates.xrot[i].dot(self.vec) - 0.5 * np.sin(0.5 * angle) * self.vec

    # state.py:142-149
    def yrot(self, angle, i):
        self.vec = np.sin(0.5 * angle) * self.gates.yrot[i].dot(self.vec) + np.cos(0.5 * angle) * self.vec

    def dyrot(self, angle, i):
        self.vec = 0.5 * np.cos(0.5 * angle) * self.gates.yrot[i].dot(self.vec) - 0.5 * np.sin(0.5 * angle) * self.vec

    # state.py:168-175
    def zrot(self, angle, i):
        self.vec = np.exp(-0.5j * angle) * self.gates.zrot_pos[i] * self.vec + \
            np.exp(0.5j * angle) * self.gates.zrot_neg[i] * self.vec

    def dzrot(self, angle, i):
        self.vec = -0.5j * np.exp(-0.5j * angle) * self.gates.zrot_pos[i] * self.vec + \
            0.5j * np.exp(0.5j * angle) * self.gates.zrot_neg[i] * self.vec

    # state.py:243-251
    def cnot_ladder(self, stacking):
        self.vec = self.gates.cnot_ladder[stacking].dot(self.vec)

    def multiply_matrix(self, matrix):
        self.vec = matrix.dot(self.vec)

    # state.py:299-301
    def exp_ham_classical(self, angle):
        self.vec *= np.exp(-1.0j * angle * self.gates.classical_ham)

    # state.py:309-311
    def exp_ham_classical_component(self, angle, i):
        self.vec *= np.exp(-1.0j * angle * self.gates.classical_ham_components[i])

    # state.py:121-123
    def x_summed(self):
        self.vec = self.gates.x_summed.dot(self.vec)

    # state.py:319-321
    def ham_classical(self):
        self.vec *= -1.0j * self.gates.classical_ham


class Observable:
    """Pauli-sum observable with the constructor the circuit code uses
    (``base.py:12``); matrix assembly follows ``observable.py:34-73``."""

    def __init__(self, qnum, observable, store_components=False):
        self.qnum = qnum
        self.info = observable
        self.store_components = store_components
        for v in observable.values():
            for s in np.shape(v):
                if s != qnum:
                    raise ValueError("Inconsistent shapes in observable dictionary.")
        n = qnum
        self.matrix = sp.csr_matrix((2 ** n, 2 ** n), dtype=complex)
        comps, weights = [], []
        for key, op in (("x", _X), ("y", _Y), ("z", _Z)):
            if key in observable and observable[key] is not None:
                for q, w in enumerate(observable[key]):
                    if w is not None:
                        if abs(w) < 1e-15:
                            warnings.warn("Weight in observable {} is zero or almost zero.".format(key))
                        m = w * _embed(n, q, op)
                        self.matrix = self.matrix + m
                        comps.append(m)
                        weights.append(w)
        if "zz" in observable:
            zz = observable["zz"]
            for i in range(n):
                for j in range(i + 1):
                    if zz[i, j] is not None:
                        raise ValueError("zz of observable should be upper triangular.")
                for j in range(i + 1, n):
                    if zz[i, j] is not None:
                        m = zz[i, j] * _embed2(n, i, _Z, j, _Z)
                        self.matrix = self.matrix + m
                        comps.append(m)
                        weights.append(zz[i, j])
        self.matrix = self.matrix.asformat("csr")
        if store_components:
            self.num_components = len(weights)
            self.component_array = comps
            self.weight_distribution = np.array(weights) / np.sum(weights)

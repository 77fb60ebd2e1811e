"""QAOA circuit on the GB300 kernels (``qradient/circuit_logic/qaoa.py``).

``Qaoa(qubit_number, observable, layer_number)``; ``run_expec_val(betas,
gammas, ...)`` (:23-38) and ``grad_run(betas, gammas, ...)`` (:40-70) with
layer i = exp(-i gamma_i C) then Rx(beta_i) on every qubit, starting from
|+..+>.  C is the diagonal of the observable's Z / ZZ terms
(state.py:261-297); for MaxCut (``MaxCut.to_observable``) it is an integer
table.  ``sample(shot_num, seed)`` draws basis states from |psi|^2 of the
last run (the shot sampler of qaoa.py:196-198, with a Philox stream).
"""
import ctypes

import numpy as np

from .. import _lib, _native
from .base import ParametrizedCircuit


class _Gates:
    """Attribute holder mirroring ``state.gates`` (qaoa.py:11-14)."""

    def __init__(self, circuit):
        self._c = circuit

    @property
    def sample_grad(self, betas, gammas, shot_num=1, hide_progbar=True, exact_expec_val=True, ini_state=None):
        """A stub in the reference too (qaoa.py:72-81): warns and returns None."""
        import warnings

        warnings.warn("Not implemented yet.")

    def grad_run_tensors(self, params, ini_state=None, out=None):
        """Device-side grad_run: params [p, 2] (beta, gamma) as a tensor or
        array; returns (E tensor[1], grad tensor[2p]) without host copies."""
        self._maybe_tune("grad")
        nat = self.native()
        return nat.grad(params, self._dtype_code, self._device(), self._grad_op(nat), ini_state=ini_state, out=out)

    def classical_ham(self):
        return self._c.classical_ham()


class Qaoa(ParametrizedCircuit):
    def __init__(self, qubit_number, observable, layer_number, **kwargs):
        ParametrizedCircuit.init(self, qubit_number, observable, **kwargs)
        kind = self.observable.terms[0]
        if np.any(kind < _lib.QG_PAULI_Z):
            import warnings

            warnings.warn("Non-classical observable component found. Only 'z' and 'zz' are accepted in this method.")
        self.lnum = int(layer_number)
        if self.lnum < 0:
            raise ValueError("layer_number must be non-negative")
        self.state.gates = _Gates(self)
        self.has_loaded_eigensystem = False

    def native(self):
        if self._native is None:
            self._native = self._apply_tuning(_native.NativeCircuit.qaoa(self.qnum, self.lnum,
                                                                         self.observable.terms))
        return self._native

    def __check_parameters(self, betas, gammas):
        betas = np.asarray(betas, dtype=np.float64).reshape(-1)
        gammas = np.asarray(gammas, dtype=np.float64).reshape(-1)
        if betas.size != self.lnum or gammas.size != self.lnum:
            raise ValueError("Wrong amount of parameters. Expected {} and {}, found {} and {}.".format(
                self.lnum, self.lnum, betas.size, gammas.size))
        return np.stack([betas, gammas], axis=1)

    def run_expec_val(self, betas, gammas, hide_progbar=True, exact_expec_val=True, shot_num=1, ini_state=None):
        """Forward run and <psi|O|psi> (qaoa.py:23-38)."""
        self._maybe_tune("run")
        params = self.__check_parameters(betas, gammas)
        nat = self.native()
        e, st = nat.run(params, self._dtype_code, self._device(), ini_state=ini_state, want_state=True)
        self.state.tensor = st
        if not exact_expec_val:
            return self.sample_expec_val(shot_num)
        return float(e.item())

    def grad_run(self, betas, gammas, hide_progbar=True, ini_state=None):
        """E and grad [p, 2] (column 0: beta, column 1: gamma) (qaoa.py:40-70)."""
        self._maybe_tune("grad")
        params = self.__check_parameters(betas, gammas)
        nat = self.native()
        op = self._grad_op(nat)
        e, g = nat.grad(params, self._dtype_code, self._device(), op, ini_state=ini_state)
        return float(e.item()), g.reshape(self.lnum, 2).cpu().numpy()

    def sample_grad(self, betas, gammas, shot_num=1, hide_progbar=True, exact_expec_val=True, ini_state=None):
        """A stub in the reference too (qaoa.py:72-81): warns and returns None."""
        import warnings

        warnings.warn("Not implemented yet.")

    def grad_run_tensors(self, params, ini_state=None, out=None):
        """Device-side grad_run: params [p, 2] (beta, gamma) as a tensor or
        array; returns (E tensor[1], grad tensor[2p]) without host copies."""
        self._maybe_tune("grad")
        nat = self.native()
        return nat.grad(params, self._dtype_code, self._device(), self._grad_op(nat), ini_state=ini_state, out=out)

    def classical_ham(self):
        """The cost diagonal C(x) as float64 (state.py:261-297)."""
        import torch

        kind, q0, q1, w = self.observable.diagonal_terms()
        dev = self._device()
        N = 2 ** self.qnum
        zz = kind == _lib.QG_PAULI_ZZ
        if np.all(zz) and np.all(w == 1.0):
            t = maxcut_table(self.qnum, np.stack([q0, q1], axis=1), device=dev)
            return t.cpu().numpy().astype(np.float64)
        # general weights: sum of weighted sign patterns on the host
        idx = np.arange(N, dtype=np.int64)
        c = np.zeros(N)
        for k, a, b, wt in zip(kind, q0, q1, w):
            s = (idx >> (self.qnum - 1 - a)) & 1
            if k == _lib.QG_PAULI_ZZ:
                s = s ^ ((idx >> (self.qnum - 1 - b)) & 1)
            c += np.where(s == 1, -wt, wt)
        return c

    def sample(self, shot_num, seed=0, offset=0):
        """Basis-state indices drawn from |psi|^2 of the last run_expec_val."""
        import torch

        if self.state.tensor is None:
            raise RuntimeError("no state: call run_expec_val first")
        return sample_state(self.state.tensor, shot_num, seed=seed, offset=offset)


def maxcut_table(n, edges, device=None):
    """Integer MaxCut / ZZ table sum_{(i,j)} z_i z_j as an int32 device tensor."""
    import torch

    dev = _native.require_cuda(device)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
    out = torch.empty(2 ** n, dtype=torch.int32, device=dev)
    _lib.check(_lib.load().qg_maxcut_table(n, len(e), e.ctypes.data_as(ctypes.c_void_p), _native.ptr(out),
                                           _native.stream_handle(dev)))
    return out


def sample_state(state, shot_num, seed=0, offset=0):
    """Draw shot_num basis indices from |state|^2 (device tensor) with Philox."""
    import torch

    dev = state.device
    n = int(state.numel()).bit_length() - 1
    code = _native.dtype_code(state.dtype)
    need = ctypes.c_size_t(0)
    lib = _lib.load()
    _lib.check(lib.qg_sample_workspace_size(n, ctypes.byref(need)))
    ws = torch.empty(max(need.value, 8), dtype=torch.uint8, device=dev)
    out = torch.empty(max(int(shot_num), 1), dtype=torch.int64, device=dev)
    _lib.check(lib.qg_sample(n, code, _native.ptr(state.contiguous()), int(shot_num), int(seed), int(offset),
                             _native.ptr(ws), ws.numel(), _native.ptr(out), _native.stream_handle(dev)))
    return out[: int(shot_num)]

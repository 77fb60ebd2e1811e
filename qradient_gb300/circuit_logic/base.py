"""Common part of the parametrised circuits (qradient/circuit_logic/base.py)."""
import numpy as np

from .. import _lib, _native
from ..physical_components import Observable, State


class ParametrizedCircuit:
    """Parent class (base.py:7-20).  Holds the qubit number, the observable,
    the device state and the options of the GB300 path:

    dtype      'complex128' (default, as the reference) or 'complex64'
    device     CUDA device (default: current)
    grad_mode  'auto' (default), 'history' or 'uncompute'
    autotune   False (default) or True: time the kernel variants for this
               circuit shape on first use (qradient_gb300.tuning)
    """

    def init(self, qubit_number, observable, use_observable_components=False, **kwargs):
        if int(qubit_number) != qubit_number or qubit_number < 1:
            raise ValueError("qubit_number must be a positive integer")
        self.qnum = int(qubit_number)
        self.state = State(self.qnum)
        self.observable = Observable(self.qnum, observable, store_components=use_observable_components)
        self.dtype = kwargs.get("dtype", "complex128")
        self._dtype_code = _native.dtype_code(self.dtype)
        self.device = kwargs.get("device", None)
        self.grad_mode = kwargs.get("grad_mode", "auto")
        self.has_loaded_projectors = False
        self._native = None
        self._native_key = None
        self._weight_cache = {}
        self.autotune = bool(kwargs.get("autotune", False))
        self._tuning = {}  # dtype code -> (tile_bits, ctas_per_sm)

    def _apply_tuning(self, nat):
        for dt, v in self._tuning.items():
            if not isinstance(dt, int):
                continue
            t, c, f = v
            _lib.check(_lib.load().qg_set_tuning(nat._h, dt, int(t), int(c), int(f)))
        return nat

    def set_tuning(self, tile_bits=0, ctas_per_sm=0, flags=0, dtype=None):
        """Fix the sweep path's fusion depth, CTAs per SM and forward kernel
        (QG_TUNE_* flags); 0 keeps the default."""
        dt = self._dtype_code if dtype is None else _native.dtype_code(dtype)
        self._tuning[dt] = (int(tile_bits), int(ctas_per_sm), int(flags))
        if self._native is not None:
            self._apply_tuning(self._native)

    def _maybe_tune(self, op):
        if self.autotune and ("tuned", self._dtype_code, op) not in self._tuning:
            from .. import tuning

            r = tuning.tune_circuit(self, op=op)
            self._tuning[self._dtype_code] = (r["tile_bits"], r["ctas_per_sm"], r.get("flags", 0))
            self._tuning[("tuned", self._dtype_code, op)] = r
            self._apply_tuning(self.native())

    def _device(self):
        return _native.require_cuda(self.device)

    def expec_val(self):
        """<psi|O|psi> of the last final state (base.py:17-20)."""
        if self.state.tensor is None:
            raise RuntimeError("no state: run the circuit first")
        v = self.state.vec
        return float(np.vdot(v, self.observable.matrix.dot(v)).real)

    # ------------------------------------------------------------ finite shots
    def _weights(self, dev):
        key = str(dev)
        w = self._weight_cache.get(key)
        if w is None:
            import torch

            w = torch.as_tensor(self.observable.terms[3], dtype=torch.float64).to(dev)
            self._weight_cache[key] = w
        return w

    @staticmethod
    def _check_shots(shot_num):
        if int(shot_num) != shot_num or shot_num < 1:
            raise ValueError("shot_num must be a positive integer, got {}".format(shot_num))
        return int(shot_num)

    @staticmethod
    def _shot_seed(seed):
        """Philox key: given, or drawn from numpy's global RNG (so that
        numpy.random.seed makes runs repeatable, as for the reference)."""
        if seed is None:
            return int(np.random.randint(0, 2 ** 62, dtype=np.int64))
        return int(seed) & ((1 << 64) - 1)

    def _state_on_device(self):
        if self.state.tensor is None:
            raise RuntimeError("no state: run the circuit first")
        import torch

        dev = self._device()
        t = self.state.tensor
        if t.device != dev or t.dtype != _native.torch_dtype(self._dtype_code):
            t = t.to(device=dev, dtype=_native.torch_dtype(self._dtype_code)).contiguous()
        return t

    def pauli_expectations(self, state=None):
        """<P_k> (unweighted) of every observable term on the device, for
        `state` or the last final state, in the observable's term order."""
        import torch

        dev = self._device()
        st = self._state_on_device() if state is None else state
        out = torch.empty(max(self.observable.num_components, 1), dtype=torch.float64, device=dev)
        self.native().pauli_expectations_into(st, self._dtype_code, dev, out)
        return out[: self.observable.num_components]

    def sample_expec_val(self, shot_num, seed=None):
        """Projector-shot estimate of <O> on the last final state
        (base.py:22-33): shot_num +-w_k outcomes per term, p = (1 + <P_k>) / 2."""
        import torch

        shot_num = self._check_shots(shot_num)
        e = self.pauli_expectations()
        total = torch.empty(1, dtype=torch.float64, device=e.device)
        _native.projector_shots(e.reshape(1, -1), self._weights(e.device), shot_num, self._shot_seed(seed),
                                total=total)
        return float(total.item())

    def sample_component_expec_val(self, shot_num, component, seed=None):
        """Projector-shot estimate of the single term w_k P_k (base.py:35-46)."""
        import torch

        shot_num = self._check_shots(shot_num)
        k = int(component)
        if not 0 <= k < self.observable.num_components:
            raise IndexError("component {} out of range".format(component))
        e = self.pauli_expectations()
        total = torch.empty(1, dtype=torch.float64, device=e.device)
        _native.projector_shots(e[k:k + 1].reshape(1, 1), self._weights(e.device)[k:k + 1], shot_num,
                                self._shot_seed(seed), total=total)
        return float(total.item())

    def _grad_op(self, native):
        return _native.choose_grad_op(native, self._dtype_code, self._device(), self.grad_mode)

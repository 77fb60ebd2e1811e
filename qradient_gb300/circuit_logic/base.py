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

    def _device(self):
        return _native.require_cuda(self.device)

    def expec_val(self):
        """<psi|O|psi> of the last final state (base.py:17-20)."""
        if self.state.tensor is None:
            raise RuntimeError("no state: run the circuit first")
        v = self.state.vec
        return float(np.vdot(v, self.observable.matrix.dot(v)).real)

    def sample_expec_val(self, shot_num):
        raise NotImplementedError("finite-shot projector estimates (base.py:22-33) are not part of the GB300 path; "
                                  "use exact_expec_val=True or Qaoa.sample for basis-state shots")

    def _grad_op(self, native):
        return _native.choose_grad_op(native, self._dtype_code, self._device(), self.grad_mode)

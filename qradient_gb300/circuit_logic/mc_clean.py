"""McClean random-Pauli-rotation circuit on the GB300 kernels.

Same constructor and methods as ``qradient/circuit_logic/mc_clean.py``:
``McClean(qubit_number, observable, layer_number, use_observable_components,
axes=, angles=)``, ``run_expec_val`` (:27-45), ``grad_run`` (:47-78) and
``grad_run_with_component_sampling`` (:80-115).
Each layer applies the entangler, then one Pauli rotation per qubit with the
axis ``axes[i, q]`` (0 X, 1 Y, 2 Z) and angle ``angles[i, q]``; the circuit
starts from Ry(pi/4) on every qubit of |0..0> (or of ``ini_state``).

Extra keyword arguments (not in the reference):
  entangler  'cnot' (default: the reference's CNOT ladder, state.py:209-251),
             'cz' (CZ on neighbours) or None
  placement  'before' (default, as the reference) or 'after' the rotations
  dtype, device, grad_mode  see ParametrizedCircuit
"""
import numpy as np

from .. import _lib, _native
from .base import ParametrizedCircuit

_ENT = {"cnot": _lib.QG_ENT_CNOT_LADDER, "cz": _lib.QG_ENT_CZ_LADDER, None: _lib.QG_ENT_NONE,
        "none": _lib.QG_ENT_NONE}
_PLACE = {"before": _lib.QG_PLACE_BEFORE, "after": _lib.QG_PLACE_AFTER}


class McClean(ParametrizedCircuit):
    def __init__(self, qubit_number, observable, layer_number, use_observable_components=False, **kwargs):
        ParametrizedCircuit.init(self, qubit_number, observable, use_observable_components, **kwargs)
        self.lnum = int(layer_number)
        if self.lnum < 0:
            raise ValueError("layer_number must be non-negative")
        # defaults drawn from the global numpy RNG exactly as mc_clean.py:13-14
        default_axes = (3 * np.random.rand(self.lnum, self.qnum)).astype("int")
        default_angles = 2 * np.pi * np.random.rand(self.lnum, self.qnum)
        self.axes = kwargs.get("axes", default_axes)
        self.angles = kwargs.get("angles", default_angles)
        ent = kwargs.get("entangler", "cnot")
        if ent not in _ENT:
            raise ValueError("entangler must be 'cnot', 'cz' or None")
        self.entangler = ent
        placement = kwargs.get("placement", "before")
        if placement not in _PLACE:
            raise ValueError("placement must be 'before' or 'after'")
        self.placement = placement
        self.has_loaded_eigensystem = False
        self.has_loaded_component_eigensystems = False

    # ------------------------------------------------------------ plumbing
    def native(self):
        """The compiled circuit for the current axes (rebuilt when they change)."""
        axes = np.asarray(self.axes)
        if axes.shape != (self.lnum, self.qnum):
            raise ValueError("axes must have shape ({}, {})".format(self.lnum, self.qnum))
        bad = axes[(axes < 0) | (axes > 2)] if axes.size else axes
        if bad.size:
            raise ValueError("Invalid axis {}".format(bad.flat[0]))
        key = axes.astype(np.int32).tobytes()
        if self._native is None or self._native_key != key:
            self._native = _native.NativeCircuit.mcclean(self.qnum, axes, self.observable.terms,
                                                         _ENT[self.entangler], _PLACE[self.placement])
            self._native_key = key
        return self._native

    def _angles(self):
        a = self.angles
        try:
            import torch

            if isinstance(a, torch.Tensor):
                return a.detach().to(torch.float64)
        except ImportError:
            pass
        a = np.asarray(a, dtype=np.float64)
        if a.shape != (self.lnum, self.qnum):
            raise ValueError("angles must have shape ({}, {})".format(self.lnum, self.qnum))
        return a

    # ------------------------------------------------------------ reference API
    def run_expec_val(self, hide_progbar=True, exact_expec_val=True, shot_num=1, ini_state=None):
        """Run the circuit and return <psi|O|psi> (mc_clean.py:27-45)."""
        if not exact_expec_val:
            return self.sample_expec_val(shot_num)
        nat = self.native()
        dev = self._device()
        e, st = nat.run(self._angles(), self._dtype_code, dev, ini_state=ini_state, want_state=True)
        self.state.tensor = st
        return float(e.item())

    def grad_run(self, hide_progbar=True, ini_state=None):
        """Expectation value and the full adjoint gradient [L, n] (mc_clean.py:47-78)."""
        nat = self.native()
        dev = self._device()
        op = self._grad_op(nat)
        e, g = nat.grad(self._angles(), self._dtype_code, dev, op, ini_state=ini_state)
        return float(e.item()), g.reshape(self.lnum, self.qnum).cpu().numpy()

    def grad_run_tensors(self, angles=None, ini_state=None, out=None):
        """Device-side grad_run: (E tensor[1], grad tensor[L*n]) without host copies."""
        nat = self.native()
        dev = self._device()
        op = self._grad_op(nat)
        return nat.grad(self._angles() if angles is None else angles, self._dtype_code, dev, op,
                        ini_state=ini_state, out=out)

    def _sample_component(self):
        """The term index drawn as at mc_clean.py:102: numpy's global RNG,
        probabilities w_k / sum(w) (observable.py:75-79)."""
        obs = self.observable
        if not obs.store_components:
            raise AttributeError("component sampling needs McClean(..., use_observable_components=True)")
        return int(np.random.choice(np.arange(obs.num_components), p=obs.weight_distribution))

    def grad_run_with_component_sampling(self, hide_progbar=True, ini_state=None):
        """Full E and the gradient of one sampled term w_k P_k (mc_clean.py:80-115)."""
        k = self._sample_component()
        nat = self.native()
        dev = self._device()
        e, g = nat.grad(self._angles(), self._dtype_code, dev, self._grad_op(nat), ini_state=ini_state, component=k)
        return float(e.item()), g.reshape(self.lnum, self.qnum).cpu().numpy()

    def grad_run_with_component_sampling_tensors(self, angles=None, ini_state=None, out=None):
        """Device-side grad_run_with_component_sampling (the component is drawn on the host)."""
        k = self._sample_component()
        nat = self.native()
        dev = self._device()
        return nat.grad(self._angles() if angles is None else angles, self._dtype_code, dev, self._grad_op(nat),
                        ini_state=ini_state, out=out, component=k)

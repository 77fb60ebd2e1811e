"""McClean random-Pauli-rotation circuit on the GB300 kernels.

Same constructor and methods as ``qradient/circuit_logic/mc_clean.py``:
``McClean(qubit_number, observable, layer_number, use_observable_components,
axes=, angles=)``, ``run_expec_val`` (:27-45), ``grad_run`` (:47-78),
``grad_run_with_component_sampling`` (:80-115) and the parameter-shift
``sample_grad`` / ``sample_grad_with_component_sampling`` (:117-205).
Each layer applies the entangler, then one Pauli rotation per qubit with the
axis ``axes[i, q]`` (0 X, 1 Y, 2 Z) and angle ``angles[i, q]``; the circuit
starts from Ry(pi/4) on every qubit of |0..0> (or of ``ini_state``).

Extra keyword arguments (not in the reference):
  entangler  'cnot' (default: the reference's CNOT ladder, state.py:209-251),
             'cnot_periodic' (its periodic form, load_cnot_ladder(periodic=True):
             CNOT(n-1, 0) joins the odd pairs; even n only), 'cz' (CZ on
             neighbours) or None
  placement  'before' (default, as the reference) or 'after' the rotations
  dtype, device, grad_mode  see ParametrizedCircuit
"""
import numpy as np
import torch

from .. import _lib, _native
from .base import ParametrizedCircuit

_ENT = {"cnot": _lib.QG_ENT_CNOT_LADDER, "cz": _lib.QG_ENT_CZ_LADDER, None: _lib.QG_ENT_NONE,
        "none": _lib.QG_ENT_NONE, "cnot_periodic": _lib.QG_ENT_CNOT_LADDER_PERIODIC}
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
            raise ValueError("entangler must be 'cnot', 'cnot_periodic', 'cz' or None")
        if ent == "cnot_periodic" and self.qnum % 2:
            # state.py:210-214
            raise ValueError(("CNOT gates in a ladder structure with periodic boundaries",
                              "are ambiguous for uneven number of qubits."))
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
            self._native = self._apply_tuning(_native.NativeCircuit.mcclean(
                self.qnum, axes, self.observable.terms, _ENT[self.entangler], _PLACE[self.placement]))
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
        """Run the circuit and return <psi|O|psi> (mc_clean.py:27-45), or its
        projector-shot estimate when exact_expec_val is False."""
        self._maybe_tune("run")
        nat = self.native()
        dev = self._device()
        e, st = nat.run(self._angles(), self._dtype_code, dev, ini_state=ini_state, want_state=True)
        self.state.tensor = st
        if not exact_expec_val:
            return self.sample_expec_val(shot_num)
        return float(e.item())

    def grad_run(self, hide_progbar=True, ini_state=None):
        """Expectation value and the full adjoint gradient [L, n] (mc_clean.py:47-78)."""
        self._maybe_tune("grad")
        nat = self.native()
        dev = self._device()
        op = self._grad_op(nat)
        e, g = nat.grad(self._angles(), self._dtype_code, dev, op, ini_state=ini_state)
        return float(e.item()), g.reshape(self.lnum, self.qnum).cpu().numpy()

    def grad_run_tensors(self, angles=None, ini_state=None, out=None):
        """Device-side grad_run: (E tensor[1], grad tensor[L*n]) without host copies."""
        self._maybe_tune("grad")
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

    # ------------------------------------------------------------ parameter shift
    def sample_grad(self, hide_progbar=True, shot_num=1, exact_expec_val=True, ini_state=None, seed=None):
        """Parameter-shift gradient with projector shots (mc_clean.py:117-156).

        grad[i, q] = (o+ - o-) / 2 with o+- the shot estimate of <O> after
        rotating qubit q of layer i by a further +-pi/2.  All rotations of a
        layer commute, so that state is the full circuit with angle
        angles[i, q] +- pi/2; the 2 L n shifted circuits run as forward
        passes on the device -- in one batched launch when the circuit fits
        the shared-memory kernel (complex64 n <= 14, complex128 n <= 13),
        else one sweep-path run each -- with every term's <P_k> on the final
        state, and one projector-shot launch draws every estimate.
        shot_num=None gives the exact parameter-shift gradient (infinitely
        many shots).  Shots are Philox draws keyed by `seed` (default: drawn
        from numpy's global RNG)."""
        return self._shift_grad(shot_num, exact_expec_val, ini_state, seed, False)

    def sample_grad_with_component_sampling(self, hide_progbar=True, shot_num=1, exact_expec_val=True,
                                            ini_state=None, seed=None):
        """sample_grad with one observable term per (layer, qubit), drawn
        with numpy.random.choice over w_k / sum(w) as mc_clean.py:187, and
        o+- the shot estimate of that term w_k P_k alone (:195-202)."""
        return self._shift_grad(shot_num, exact_expec_val, ini_state, seed, True)

    def _shift_grad(self, shot_num, exact_expec_val, ini_state, seed, component_sampling):
        if shot_num is not None:
            shot_num = self._check_shots(shot_num)
        nat = self.native()
        dev = self._device()
        dt = self._dtype_code
        L, n = self.lnum, self.qnum
        K = self.observable.num_components
        # forward run: E (exact or sampled) and the final state
        expec_val = self.run_expec_val(exact_expec_val=exact_expec_val, shot_num=shot_num or 1, ini_state=ini_state)
        comps = [self._sample_component() for _ in range(L * n)] if component_sampling else None
        base = torch.as_tensor(self._angles(), dtype=torch.float64).reshape(-1).to(dev)
        rows = 2 * L * n
        if rows == 0:
            return expec_val, np.zeros((L, n))
        shifted = base.repeat(rows, 1)
        idx = torch.arange(L * n, device=dev)
        shifted[2 * idx, idx] += np.pi / 2
        shifted[2 * idx + 1, idx] -= np.pi / 2
        need_terms = shot_num is not None or component_sampling
        expec = torch.empty((rows, max(K, 1)), dtype=torch.float64, device=dev)
        from ..batched import CLUSTER_MAX, Batch

        if ini_state is None and n <= CLUSTER_MAX[dt]:
            # the 2 L n shifted circuits as one batched launch: each a whole
            # forward run in shared memory, with its energy and (for shots)
            # every term's <P_k>
            b = Batch(device=dev, dtype=dt, grad=False, use_graph=False, term_expectations=need_terms)
            for _ in range(rows):
                b.add(self)
            b.finalize()
            b.params_flat[: rows * L * n].copy_(shifted.reshape(-1))
            b.execute()
            energies = b.expec[:rows]
            if need_terms and K:
                expec[:, :K] = b.term_expec_flat[: rows * K].reshape(rows, K)
        else:
            ini = nat.state_tensor(ini_state, dt, dev)
            ws = nat.workspace(dt, _lib.QG_OP_RUN, dev)
            energies = torch.empty(rows, dtype=torch.float64, device=dev)
            state = torch.empty(2 ** n, dtype=_native.torch_dtype(dt), device=dev)
            for r in range(rows):
                nat.run_into(shifted[r], dt, dev, ini, ws, energies[r:r + 1], state if need_terms else None)
                if need_terms and K:
                    nat.pauli_expectations_into(state, dt, dev, expec[r])
        w = self._weights(dev)
        if component_sampling:
            k = torch.as_tensor(np.repeat(comps, 2), device=dev)
            r_idx = torch.arange(rows, device=dev)
            if shot_num is None:
                vals = w[k] * expec[r_idx, k]
            else:
                term_est = torch.empty((rows, K), dtype=torch.float64, device=dev)
                _native.projector_shots(expec[:, :K], w, shot_num, self._shot_seed(seed), term_est=term_est)
                vals = term_est[r_idx, k]
        elif shot_num is None:
            vals = energies
        else:
            vals = torch.empty(rows, dtype=torch.float64, device=dev)
            _native.projector_shots(expec[:, :K], w, shot_num, self._shot_seed(seed), total=vals)
        v = vals.reshape(L * n, 2)
        grad = (0.5 * (v[:, 0] - v[:, 1])).reshape(L, n)
        return expec_val, grad.cpu().numpy()

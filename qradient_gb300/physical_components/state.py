"""Device-resident statevector holder (counterpart of
``qradient/physical_components/state.py``'s ``State.vec``)."""
import numpy as np


class State:
    """Holds the last final state a circuit produced, on the device.

    ``vec`` copies it to the host as a numpy array, as the reference's
    ``State.vec`` (state.py:25) is read by callers."""

    def __init__(self, qubit_number):
        self.qnum = qubit_number
        self.tensor = None
        self.gates = None

    @property
    def vec(self):
        if self.tensor is None:
            return None
        return self.tensor.detach().cpu().numpy()

    @vec.setter
    def vec(self, value):
        import torch

        self.tensor = None if value is None else torch.as_tensor(np.asarray(value))

    def norm_error(self):
        """1 - ||vec|| (state.py:331-332)."""
        v = self.vec
        return 1.0 - float(np.linalg.norm(v))

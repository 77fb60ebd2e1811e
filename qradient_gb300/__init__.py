"""GB300-native statevector run / adjoint grad_run path of qradient.

Drop-in counterparts of ``qradient.circuit_logic.McClean`` and ``Qaoa``;
every state update runs in hand-written sm_103a CUDA kernels
(``libqgrad.so``, C ABI in ``include/qgrad.h``) on PyTorch-owned device
memory.
"""
from . import circuit_logic, physical_components
from .circuit_logic import McClean, Qaoa
from .physical_components import Observable, State

__all__ = ["McClean", "Qaoa", "Observable", "State", "circuit_logic", "physical_components"]

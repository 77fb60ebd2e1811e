"""Observable and state objects of the GB300 statevector path
(counterparts of qradient/physical_components)."""
from .observable import Observable
from .state import State

__all__ = ["Observable", "State"]

"""Drop-in counterparts of qradient.circuit_logic (McClean, Qaoa) running on
the GB300 statevector kernels."""
from .mc_clean import McClean
from .qaoa import Qaoa

__all__ = ["McClean", "Qaoa"]

"""ctypes binding of ``libqgrad.so`` (declarations in ``include/qgrad.h``).

The library is built in-tree (``qradient_gb300/build.py``).  There is no
fallback: if the library is missing or fails to load, every call raises.
"""
import ctypes
import os

from . import build as _build

QG_OK, QG_ERR_INVALID, QG_ERR_CUDA, QG_ERR_WORKSPACE, QG_ERR_UNSUPPORTED, QG_ERR_HOST_MEMORY = range(6)
QG_C128, QG_C64 = 0, 1
QG_ENT_NONE, QG_ENT_CNOT_LADDER, QG_ENT_CZ_LADDER, QG_ENT_CNOT_LADDER_PERIODIC = 0, 1, 2, 3
QG_PLACE_BEFORE, QG_PLACE_AFTER = 0, 1
QG_PAULI_X, QG_PAULI_Y, QG_PAULI_Z, QG_PAULI_ZZ = 0, 1, 2, 3
QG_OP_RUN, QG_OP_GRAD_HISTORY, QG_OP_GRAD_UNCOMPUTE = 0, 1, 2
QG_TUNE_FWD_PIPELINED, QG_TUNE_FWD_PLAIN = 1, 2

# every symbol include/qgrad.h declares, with its ctypes signature
_P = ctypes.c_void_p
_I = ctypes.c_int
_SZ = ctypes.c_size_t
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
SIGNATURES = {
    "qg_mcclean_create": (_I, [_I, _I, _P, _I, _I, _I, _P, _P, _P, _P, ctypes.POINTER(_P)]),
    "qg_qaoa_create": (_I, [_I, _I, _I, _P, _P, _P, _P, ctypes.POINTER(_P)]),
    "qg_destroy": (None, [_P]),
    "qg_num_params": (_I, [_P, ctypes.POINTER(_I)]),
    "qg_workspace_size": (_I, [_P, _I, _I, ctypes.POINTER(_SZ)]),
    "qg_run": (_I, [_P, _I, _P, _P, _P, _SZ, _P, _P, _P]),
    "qg_grad": (_I, [_P, _I, _I, _P, _P, _P, _SZ, _P, _P, _P]),
    "qg_grad_component": (_I, [_P, _I, _I, _P, _P, _I, _P, _SZ, _P, _P, _P]),
    "qg_maxcut_table": (_I, [_I, _I, _P, _P, _P]),
    "qg_sample_workspace_size": (_I, [_I, ctypes.POINTER(_SZ)]),
    "qg_sample": (_I, [_I, _I, _P, _I64, _U64, _U64, _P, _SZ, _P, _P]),
    "qg_qaoa_cost_terms": (_I, [_I, _I, _P, _P, _P, _P, _I, _P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(_I)]),
    "qg_batch_workspace_size": (_I, [ctypes.POINTER(_SZ)]),
    "qg_batch_launch": (_I, [_I, _P, _I, _I, _I, _P, _SZ, _P]),
    "qg_grad_noalloc": (_I, [_P, _I, _P, _P, _P, _P, _P]),
    "qg_set_tuning": (_I, [_P, _I, _I, _I, _I]),
    "qg_get_tuning": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "qg_pauli_workspace_size": (_I, [_P, ctypes.POINTER(_SZ)]),
    "qg_pauli_expectations": (_I, [_P, _I, _P, _P, _SZ, _P, _P]),
    "qg_projector_shots": (_I, [_I, _I, _P, _P, _I, ctypes.c_uint64, ctypes.c_uint64, _P, _P, _P]),
    "qg_adam_step": (_I, [_P, _P, _P, _P, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                          ctypes.c_double, _P, _P]),
    "qg_gd_step": (_I, [_P, _P, _I, ctypes.c_double, _P, _P]),
    "qg_plateau_step": (_I, [_P, _P, _I, _P, _P, _I, ctypes.c_double, _P, _P]),
    "qg_profile_enable": (_I, [_I]),
    "qg_profile_collect": (_I, [_I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)]),
    "qg_status_string": (ctypes.c_char_p, [_I]),
    "qg_last_error": (ctypes.c_char_p, []),
    "qg_version": (_I, []),
}

_lib = None


class QgradError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def load(build_if_missing=True):
    """Load (building first if needed) the in-tree library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libqgrad.so is not built (%s); run qradient_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status):
    """Map a qgrad status to the reference's exception types."""
    if status == QG_OK:
        return
    lib = load()
    msg = (lib.qg_last_error() or b"").decode() or lib.qg_status_string(status).decode()
    if status == QG_ERR_INVALID:
        raise ValueError(msg)
    if status == QG_ERR_HOST_MEMORY:
        raise MemoryError(msg)
    raise QgradError(status, "%s: %s" % (lib.qg_status_string(status).decode(), msg))

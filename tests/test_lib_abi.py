"""The C-ABI library builds, loads and exports every symbol include/qgrad.h
declares; host-only entry points validate their arguments (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "qgrad.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from qradient_gb300 import _lib

    lib = _lib.load()
    names = _declared()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


def test_status_strings_and_version():
    from qradient_gb300 import _lib

    lib = _lib.load()
    assert lib.qg_version() >= 1
    assert lib.qg_status_string(0) == b"ok"
    assert lib.qg_status_string(3) == b"workspace too small"


def _create(n, L, axes, kind=(3,), q0=(0,), q1=(1,), w=(1.0,), ent=1, place=0):
    from qradient_gb300 import _lib

    lib = _lib.load()
    ax = np.ascontiguousarray(axes, dtype=np.int32)
    k = np.array(kind, np.int32)
    a = np.array(q0, np.int32)
    b = np.array(q1, np.int32)
    ww = np.array(w, np.float64)
    h = ctypes.c_void_p()
    st = lib.qg_mcclean_create(n, L, ax.ctypes.data_as(ctypes.c_void_p), ent, place, len(k),
                               k.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                               b.ctypes.data_as(ctypes.c_void_p), ww.ctypes.data_as(ctypes.c_void_p),
                               ctypes.byref(h))
    return st, h


def test_create_validates_like_the_reference():
    from qradient_gb300 import _lib

    lib = _lib.load()
    st, h = _create(4, 2, np.zeros((2, 4)))
    assert st == 0 and h.value
    nparams = ctypes.c_int()
    assert lib.qg_num_params(h, ctypes.byref(nparams)) == 0 and nparams.value == 8
    for op in (0, 1, 2):
        b = ctypes.c_size_t()
        assert lib.qg_workspace_size(h, 0, op, ctypes.byref(b)) == 0 and b.value > 0
    lib.qg_destroy(h)
    # invalid axis -> QG_ERR_INVALID (mc_clean.py:391-392 raises ValueError)
    st, h = _create(4, 1, [[0, 1, 3, 0]])
    assert st == _lib.QG_ERR_INVALID and b"Invalid axis" in lib.qg_last_error()
    # zz in the lower triangle -> invalid (observable.py:57-64)
    st, h = _create(4, 1, [[0, 0, 0, 0]], q0=(2,), q1=(1,))
    assert st == _lib.QG_ERR_INVALID
    with pytest.raises(ValueError):
        _lib.check(st)
    # too many qubits -> unsupported
    st, h = _create(40, 0, np.zeros((0, 40)))
    assert st == _lib.QG_ERR_UNSUPPORTED


def test_history_needs_more_workspace_than_uncompute():
    from qradient_gb300 import _lib

    lib = _lib.load()
    st, h = _create(20, 10, np.zeros((10, 20)))
    assert st == 0
    sizes = []
    for op in (0, 1, 2):
        b = ctypes.c_size_t()
        lib.qg_workspace_size(h, 0, op, ctypes.byref(b))
        sizes.append(b.value)
    lib.qg_destroy(h)
    S = 16 * 2 ** 20
    assert sizes[0] >= S and sizes[2] >= 2 * S and sizes[1] > sizes[2]


def test_product_path_fails_loudly_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    from qradient_gb300 import McClean

    zz = np.full((3, 3), None)
    zz[0, 1] = 1.0
    c = McClean(3, {"zz": zz}, 1)
    with pytest.raises(RuntimeError, match="CUDA"):
        c.grad_run()


def test_optimiser_steps_and_component_gradient_validate_arguments():
    """Argument checks that return before any CUDA call."""
    from qradient_gb300 import _lib

    lib = _lib.load()
    P = ctypes.c_void_p
    fake = P(256)  # never dereferenced: every call below returns before a launch
    INV = _lib.QG_ERR_INVALID
    assert lib.qg_adam_step(fake, fake, fake, fake, -1, 1, 0.1, 0.9, 0.999, 1e-8, None, None) == INV
    assert lib.qg_adam_step(fake, fake, fake, fake, 4, 0, 0.1, 0.9, 0.999, 1e-8, None, None) == INV
    assert lib.qg_adam_step(fake, None, fake, fake, 4, 1, 0.1, 0.9, 0.999, 1e-8, None, None) == INV
    assert lib.qg_adam_step(None, None, None, None, 0, 1, 0.1, 0.9, 0.999, 1e-8, None, None) == 0
    assert lib.qg_gd_step(fake, fake, -2, 0.1, None, None) == INV
    assert lib.qg_gd_step(None, fake, 3, 0.1, None, None) == INV
    assert lib.qg_gd_step(None, None, 0, 0.1, None, None) == 0
    assert lib.qg_plateau_step(fake, fake, 3, None, fake, 2, 0.5, None, None) == INV
    st, h = _create(4, 2, np.zeros((2, 4)), kind=(0, 3), q0=(1, 0), q1=(1, 1), w=(0.5, 1.0))
    assert st == 0
    for k in (-1, 2):
        assert lib.qg_grad_component(h, 0, 1, fake, None, k, fake, 1 << 20, fake, fake, None) == INV
        assert b"component" in lib.qg_last_error()
    lib.qg_destroy(h)


def test_default_tile_bits_save_sweeps():
    """complex128 takes 12-bit tiles where they need one sweep per layer
    fewer than 11-bit ones (n = 20, 21, 28-30), else 11; complex64 12."""
    from qradient_gb300 import _lib

    lib = _lib.load()
    t, c, f = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    for n, want128 in ((16, 11), (19, 11), (20, 12), (21, 12), (24, 11), (27, 11), (28, 12), (30, 12), (31, 11)):
        st, h = _create(n, 1, np.zeros((1, n)))
        assert st == 0
        assert lib.qg_get_tuning(h, 0, ctypes.byref(t), ctypes.byref(c), ctypes.byref(f)) == 0
        assert t.value == want128, n
        assert lib.qg_get_tuning(h, 1, ctypes.byref(t), ctypes.byref(c), ctypes.byref(f)) == 0
        assert t.value == 12, n
        lib.qg_destroy(h)


def test_tuning_knobs_validate_and_report():
    from qradient_gb300 import _lib

    lib = _lib.load()
    st, h = _create(20, 2, np.zeros((2, 20)))
    assert st == 0
    INV = _lib.QG_ERR_INVALID
    assert lib.qg_set_tuning(h, 0, 4, 0, 0) == INV
    assert lib.qg_set_tuning(h, 0, 13, 0, 0) == INV
    assert lib.qg_set_tuning(h, 1, 5, 0, 0) == INV
    assert lib.qg_set_tuning(h, 1, 13, 0, 0) == 0
    assert lib.qg_set_tuning(h, 5, 11, 0, 0) == INV
    assert lib.qg_set_tuning(h, 0, 11, -1, 0) == INV
    assert lib.qg_set_tuning(h, 0, 11, 0, 3) == INV
    assert lib.qg_set_tuning(h, 0, 11, 0, 4) == INV
    t, c, f = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    for bits, flags in ((10, 1), (11, 2), (0, 0)):
        assert lib.qg_set_tuning(h, 0, bits, 0, flags) == 0
        assert lib.qg_get_tuning(h, 0, ctypes.byref(t), ctypes.byref(c), ctypes.byref(f)) == 0
        # default at n = 20: 12 bits, two sweeps per layer where 11 needs three
        assert t.value == (bits or 12)
        assert f.value in (1, 2) and (flags == 0 or f.value == flags)
    # history workspace holds one state per sweep: deeper fusion, fewer sweeps
    sizes = []
    for bits in (10, 12):
        lib.qg_set_tuning(h, 0, bits, 0, 0)
        b = ctypes.c_size_t()
        lib.qg_workspace_size(h, 0, 1, ctypes.byref(b))
        sizes.append(b.value)
    assert sizes[0] > sizes[1]
    lib.qg_destroy(h)
    st, h = _create(6, 1, np.zeros((1, 6)))
    assert lib.qg_set_tuning(h, 1, 12, 0, 0) == 0
    assert lib.qg_get_tuning(h, 1, ctypes.byref(t), ctypes.byref(c), None) == 0 and t.value == 6
    lib.qg_destroy(h)

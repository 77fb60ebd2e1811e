"""Python side of a native circuit handle: workspaces, dtypes, launches.

PyTorch provides device memory and streams only; every state update runs in
``libqgrad.so``.  A call on a machine without CUDA raises: there is no CPU
fallback.
"""
import ctypes

import numpy as np
import torch

from . import _lib

_DTYPES = {
    "complex128": _lib.QG_C128,
    "c128": _lib.QG_C128,
    "complex64": _lib.QG_C64,
    "c64": _lib.QG_C64,
    torch.complex128: _lib.QG_C128,
    torch.complex64: _lib.QG_C64,
    np.complex128: _lib.QG_C128,
    np.complex64: _lib.QG_C64,
}
_TORCH = {_lib.QG_C128: torch.complex128, _lib.QG_C64: torch.complex64}


def dtype_code(dtype):
    if isinstance(dtype, int) and not isinstance(dtype, bool) and dtype in (_lib.QG_C128, _lib.QG_C64):
        return dtype
    try:
        return _DTYPES[dtype]
    except (KeyError, TypeError):
        pass
    try:
        return _DTYPES[np.dtype(dtype).type]
    except (KeyError, TypeError):
        raise ValueError("unsupported dtype %r (use complex128 or complex64)" % (dtype,))


def torch_dtype(code):
    return _TORCH[code]


def require_cuda(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError("qradient_gb300 needs a CUDA GPU: the statevector path has no CPU implementation")
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("device must be a CUDA device, got %s" % device)
    return device


def stream_handle(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class NativeCircuit:
    """Owns a qg_circuit handle and the device workspaces used with it."""

    def __init__(self, handle, kind, n, layers):
        self._h = handle
        self.kind = kind
        self.n = n
        self.layers = layers
        np_ = ctypes.c_int(0)
        _lib.check(_lib.load().qg_num_params(self._h, ctypes.byref(np_)))
        self.nparams = np_.value
        self._ws = {}

    @classmethod
    def mcclean(cls, n, axes, terms, entangler, placement):
        lib = _lib.load()
        axes = _arr(axes, np.int32).reshape(-1)
        L = axes.size // n if n else 0
        kind, q0, q1, w = terms
        h = ctypes.c_void_p()
        _lib.check(lib.qg_mcclean_create(n, L, axes.ctypes.data, entangler, placement,
                                         len(kind), kind.ctypes.data,
                                         q0.ctypes.data, q1.ctypes.data,
                                         w.ctypes.data, ctypes.byref(h)))
        return cls(h, 0, n, L)

    @classmethod
    def qaoa(cls, n, p, terms):
        lib = _lib.load()
        kind, q0, q1, w = terms
        h = ctypes.c_void_p()
        _lib.check(lib.qg_qaoa_create(n, p, len(kind), kind.ctypes.data,
                                      q0.ctypes.data, q1.ctypes.data,
                                      w.ctypes.data, ctypes.byref(h)))
        return cls(h, 1, n, p)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.qg_destroy(h)
            self._h = None

    def workspace_bytes(self, dtype, op):
        b = ctypes.c_size_t(0)
        _lib.check(_lib.load().qg_workspace_size(self._h, dtype, op, ctypes.byref(b)))
        return b.value

    def workspace(self, dtype, op, device):
        key = (dtype, op, str(device))
        ws = self._ws.get(key)
        need = self.workspace_bytes(dtype, op)
        if ws is None or ws.numel() < need:
            self._ws.pop(key, None)
            ws = torch.empty(max(need, 256), dtype=torch.uint8, device=device)
            self._ws[key] = ws
        return ws

    def release_workspaces(self):
        self._ws.clear()

    def params_tensor(self, params, device):
        t = torch.as_tensor(params, dtype=torch.float64)
        if t.numel() != self.nparams:
            raise ValueError("expected %d parameters, got %d" % (self.nparams, t.numel()))
        return t.reshape(-1).to(device, non_blocking=True).contiguous()

    def state_tensor(self, state, dtype, device):
        if state is None:
            return None
        t = torch.as_tensor(state)
        if t.numel() != 2 ** self.n:
            raise ValueError("ini_state must have 2**%d entries, got %d" % (self.n, t.numel()))
        return t.reshape(-1).to(device=device, dtype=torch_dtype(dtype), non_blocking=True).contiguous()

    def run(self, params, dtype, device, ini_state=None, want_state=False, workspace=None):
        """Forward + expectation on device; returns (E tensor[1], state or None)."""
        lib = _lib.load()
        p = self.params_tensor(params, device)
        ini = self.state_tensor(ini_state, dtype, device)
        ws = workspace if workspace is not None else self.workspace(dtype, _lib.QG_OP_RUN, device)
        e = torch.empty(1, dtype=torch.float64, device=device)
        st = torch.empty(2 ** self.n, dtype=torch_dtype(dtype), device=device) if want_state else None
        _lib.check(lib.qg_run(self._h, dtype, ptr(p), ptr(ini), ptr(ws), ws.numel(), ptr(e), ptr(st),
                              stream_handle(device)))
        return e, st

    def run_into(self, params, dtype, device, ini, workspace, expec, state):
        """qg_run with caller tensors: params and ini already on the device,
        expec a 1-element float64 view, state a 2^n buffer (or None)."""
        _lib.check(_lib.load().qg_run(self._h, dtype, ptr(params), ptr(ini), ptr(workspace), workspace.numel(),
                                      ptr(expec), ptr(state), stream_handle(device)))

    def pauli_workspace(self, device):
        key = ("pauli", str(device))
        b = ctypes.c_size_t(0)
        _lib.check(_lib.load().qg_pauli_workspace_size(self._h, ctypes.byref(b)))
        ws = self._ws.get(key)
        if ws is None or ws.numel() < b.value:
            ws = torch.empty(max(b.value, 8), dtype=torch.uint8, device=device)
            self._ws[key] = ws
        return ws

    def pauli_expectations_into(self, state, dtype, device, out):
        """out[k] = <state|P_k|state> for every observable term (qg_pauli_expectations)."""
        ws = self.pauli_workspace(device)
        _lib.check(_lib.load().qg_pauli_expectations(self._h, dtype, ptr(state), ptr(ws), ws.numel(), ptr(out),
                                                     stream_handle(device)))
        return out

    def grad(self, params, dtype, device, op, ini_state=None, workspace=None, out=None, component=None):
        """Adjoint gradient on device; returns (E tensor[1], grad tensor[nparams]).

        component: index of one observable term; the gradient is then that
        term's (qg_grad_component) while E stays the full expectation."""
        lib = _lib.load()
        p = self.params_tensor(params, device)
        ini = self.state_tensor(ini_state, dtype, device)
        ws = workspace if workspace is not None else self.workspace(dtype, op, device)
        if out is None:
            e = torch.empty(1, dtype=torch.float64, device=device)
            g = torch.empty(max(self.nparams, 1), dtype=torch.float64, device=device)
        else:
            e, g = out
        if component is None:
            _lib.check(lib.qg_grad(self._h, dtype, op, ptr(p), ptr(ini), ptr(ws), ws.numel(), ptr(e), ptr(g),
                                   stream_handle(device)))
        else:
            _lib.check(lib.qg_grad_component(self._h, dtype, op, ptr(p), ptr(ini), int(component), ptr(ws),
                                             ws.numel(), ptr(e), ptr(g), stream_handle(device)))
        return e, g[: self.nparams]


def projector_shots(expec, weights, shot_num, seed, offset=0, term_est=None, total=None):
    """qg_projector_shots over rows of expectations [rows, K] (device)."""
    rows, K = expec.shape
    _lib.check(_lib.load().qg_projector_shots(rows, K, ptr(expec), ptr(weights), int(shot_num), int(seed), int(offset),
                                              ptr(term_est), ptr(total), stream_handle(expec.device)))


def choose_grad_op(circuit, dtype, device, mode="auto", budget_fraction=0.6):
    """History mode when its workspace fits in a fraction of free memory."""
    if mode == "history":
        return _lib.QG_OP_GRAD_HISTORY
    if mode == "uncompute":
        return _lib.QG_OP_GRAD_UNCOMPUTE
    if mode != "auto":
        raise ValueError("grad_mode must be 'auto', 'history' or 'uncompute'")
    need = circuit.workspace_bytes(dtype, _lib.QG_OP_GRAD_HISTORY)
    key = (dtype, _lib.QG_OP_GRAD_HISTORY, str(device))
    have = circuit._ws.get(key)
    if have is not None and have.numel() >= need:
        return _lib.QG_OP_GRAD_HISTORY
    free, _total = torch.cuda.mem_get_info(device)
    free += torch.cuda.memory_reserved(device) - torch.cuda.memory_allocated(device)
    return _lib.QG_OP_GRAD_HISTORY if need <= budget_fraction * free else _lib.QG_OP_GRAD_UNCOMPUTE

"""qg_grad_noalloc: the allocation-free gradient entry point.

It serves callers that cannot allocate device memory when they need a
gradient: a host process that owns every device allocation through its own
pool, or a real-time loop that must not allocate (cudaMalloc may
synchronise the device) after start-up.
Its scratch is a fixed static device array inside the library, so the caller
passes only inputs and outputs.  This test calls it through the C ABI twice
in a row and checks each result against qg_grad with a caller-provided
workspace, to the 1e-12 (complex128) / 1e-5 (complex64) tolerances of the
other GPU tests.  It lives in its own file so that a failure here comes
after every other test has run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grad_both(nat, params_list, dtype):
    import torch

    from qradient_gb300 import _lib
    from qradient_gb300._native import ptr, stream_handle

    lib = _lib.load()
    dev = torch.device("cuda", 0)
    ws = nat.workspace(dtype, _lib.QG_OP_GRAD_UNCOMPUTE, dev)
    out = []
    for params in params_list:
        p = torch.as_tensor(params.reshape(-1), dtype=torch.float64, device=dev)
        e_ref = torch.empty(1, dtype=torch.float64, device=dev)
        g_ref = torch.empty(nat.nparams, dtype=torch.float64, device=dev)
        _lib.check(lib.qg_grad(nat._h, dtype, _lib.QG_OP_GRAD_UNCOMPUTE, ptr(p), None, ptr(ws), ws.numel(),
                               ptr(e_ref), ptr(g_ref), stream_handle(dev)))
        e = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
        g = torch.full((nat.nparams,), np.nan, dtype=torch.float64, device=dev)
        _lib.check(lib.qg_grad_noalloc(nat._h, dtype, ptr(p), None, ptr(e), ptr(g), stream_handle(dev)))
        torch.cuda.synchronize()
        out.append((e_ref.item(), g_ref.cpu().numpy(), e.item(), g.cpu().numpy()))
    return out


def _check(out, tol):
    for e_ref, g_ref, e, g in out:
        assert abs(e - e_ref) <= tol * max(1.0, abs(e_ref))
        assert np.max(np.abs(g - g_ref)) <= tol * max(np.max(np.abs(g_ref)), 1e-300)


@pytest.mark.parametrize("dtype,tol", [(0, 1e-12), (1, 1e-5)])
def test_noalloc_matches_qg_grad_mcclean(dtype, tol):
    import torch

    from qradient_gb300 import McClean

    torch.cuda.set_device(0)
    n, L = 13, 4
    rng = np.random.default_rng(42)
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    c = McClean(n, {"zz": zz, "x": np.array([0.5] + [None] * (n - 1), dtype=object)}, L,
                axes=rng.integers(0, 3, (L, n)), angles=np.zeros((L, n)))
    nat = c.native()
    p1 = rng.uniform(0, 2 * np.pi, (L, n))
    p2 = rng.uniform(0, 2 * np.pi, (L, n))
    _check(_grad_both(nat, [p1, p2], dtype), tol)


def test_noalloc_matches_qg_grad_qaoa():
    import torch

    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    torch.cuda.set_device(0)
    n, p = 12, 3
    q = Qaoa(n, MaxCut(n, edge_set=random_regular_edges(3, n, 5)).to_observable(), p)
    rng = np.random.default_rng(7)
    a = np.stack([rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)], 1)
    b = np.stack([rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)], 1)
    _check(_grad_both(q.native(), [a, b], 0), 1e-12)


def test_noalloc_rejects_circuits_beyond_its_scratch():
    import torch

    from qradient_gb300 import McClean, _lib
    from qradient_gb300._native import ptr, stream_handle

    torch.cuda.set_device(0)
    n, L = 22, 1
    zz = np.full((n, n), None)
    zz[0, 1] = 1.0
    c = McClean(n, {"zz": zz}, L, axes=np.zeros((L, n), dtype=int), angles=np.zeros((L, n)))
    nat = c.native()
    dev = torch.device("cuda", 0)
    prm = torch.zeros(n * L, dtype=torch.float64, device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    g = torch.zeros(n * L, dtype=torch.float64, device=dev)
    lib = _lib.load()
    st = lib.qg_grad_noalloc(nat._h, 0, ptr(prm), None, ptr(e), ptr(g), stream_handle(dev))
    assert st == _lib.QG_ERR_UNSUPPORTED
    assert b"scratch" in lib.qg_last_error()

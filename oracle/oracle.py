"""ctypes front end of the CPU oracle (``oracle/qg_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` to check or time the reference's
algorithm.  The ``qradient_gb300`` product never imports this module.

The oracle restates the reference's numpy path gate by gate
(``qradient/circuit_logic/mc_clean.py:27-78``, ``qaoa.py:23-70``,
``physical_components/state.py``, ``observable.py:34-73``); see the header of
``qg_oracle.c`` for the line-by-line map.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libqg_oracle.so")

X, Y, Z, ZZ = 0, 1, 2, 3
ENT_NONE, ENT_CNOT, ENT_CZ, ENT_CNOT_PERIODIC = 0, 1, 2, 3
PLACE_BEFORE, PLACE_AFTER = 0, 1


def build(force=False):
    """Compile the oracle with gcc (OpenMP) into ``oracle/_build``."""
    src = os.path.join(HERE, "qg_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", tmp, src, "-lm"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        for name, args in {
            "qgo_mcclean_run": [I, I, P, P, I, I, I, P, P, P, P, P, P, P],
            "qgo_mcclean_grad": [I, I, P, P, I, I, I, P, P, P, P, P, P, P],
            "qgo_mcclean_grad_uncompute": [I, I, P, P, I, I, I, P, P, P, P, P, P, P],
            "qgo_qaoa_run": [I, I, P, P, I, P, P, P, P, P, P, P],
            "qgo_qaoa_grad": [I, I, P, P, I, P, P, P, P, P, P, P],
            "qgo_qaoa_grad_uncompute": [I, I, P, P, I, P, P, P, P, P, P, P],
            "qgo_maxcut_table": [I, I, P, P],
            "qgo_entangle": [I, I, I, P],
            "qgo_num_threads": [],
        }.items():
            f = getattr(_lib, name)
            f.argtypes = args
            f.restype = ctypes.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Terms:
    """Observable as parallel arrays (kind, q0, q1, w)."""

    def __init__(self, kind, q0, q1, w):
        self.kind = np.ascontiguousarray(kind, dtype=np.int32)
        self.q0 = np.ascontiguousarray(q0, dtype=np.int32)
        self.q1 = np.ascontiguousarray(q1, dtype=np.int32)
        self.w = np.ascontiguousarray(w, dtype=np.float64)

    def __len__(self):
        return len(self.kind)

    @classmethod
    def from_dict(cls, n, obs):
        """Reference observable dict ('x', 'y', 'z': length-n arrays, 'zz':
        n x n strict upper triangle; None = absent), observable.py:12-17."""
        kind, q0, q1, w = [], [], [], []
        for key, k in (("x", X), ("y", Y), ("z", Z)):
            if key in obs and obs[key] is not None:
                for q, v in enumerate(obs[key]):
                    if v is not None:
                        kind.append(k), q0.append(q), q1.append(q), w.append(float(v))
        if "zz" in obs and obs["zz"] is not None:
            zz = obs["zz"]
            for i in range(n):
                for j in range(i + 1, n):
                    if zz[i, j] is not None:
                        kind.append(ZZ), q0.append(i), q1.append(j), w.append(float(zz[i, j]))
        return cls(kind, q0, q1, w)


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


def _chk(st):
    if st != 0:
        raise ValueError("oracle status %d" % st)


def mcclean_grad(n, axes, angles, terms, entangler=ENT_CNOT, placement=PLACE_BEFORE, ini=None, uncompute=False):
    """McClean.grad_run; uncompute=True keeps one psi instead of the L+1
    stored states (for sizes whose history does not fit in host memory)."""
    axes = _c(axes, np.int32)
    angles = _c(angles, np.float64)
    L = axes.shape[0]
    ini = _c(ini, np.complex128)
    E = np.zeros(1)
    g = np.zeros((L, n))
    f = lib().qgo_mcclean_grad_uncompute if uncompute else lib().qgo_mcclean_grad
    _chk(f(n, L, _p(axes), _p(angles), entangler, placement, len(terms), _p(terms.kind), _p(terms.q0),
           _p(terms.q1), _p(terms.w), _p(ini), _p(E), _p(g)))
    return float(E[0]), g


def mcclean_run(n, axes, angles, terms, entangler=ENT_CNOT, placement=PLACE_BEFORE, ini=None, want_state=False):
    axes = _c(axes, np.int32)
    angles = _c(angles, np.float64)
    L = axes.shape[0]
    ini = _c(ini, np.complex128)
    E = np.zeros(1)
    st = np.zeros(2 ** n, dtype=np.complex128) if want_state else None
    _chk(lib().qgo_mcclean_run(n, L, _p(axes), _p(angles), entangler, placement, len(terms), _p(terms.kind),
                               _p(terms.q0), _p(terms.q1), _p(terms.w), _p(ini), _p(E), _p(st)))
    return (float(E[0]), st) if want_state else float(E[0])


def qaoa_grad(n, betas, gammas, terms, ini=None, uncompute=False):
    """Qaoa.grad_run; uncompute=True keeps one psi instead of 2p+1 states."""
    betas = _c(betas, np.float64)
    gammas = _c(gammas, np.float64)
    p = betas.shape[0]
    ini = _c(ini, np.complex128)
    E = np.zeros(1)
    g = np.zeros((p, 2))
    f = lib().qgo_qaoa_grad_uncompute if uncompute else lib().qgo_qaoa_grad
    _chk(f(n, p, _p(betas), _p(gammas), len(terms), _p(terms.kind), _p(terms.q0), _p(terms.q1), _p(terms.w),
           _p(ini), _p(E), _p(g)))
    return float(E[0]), g


def qaoa_run(n, betas, gammas, terms, ini=None, want_state=False):
    betas = _c(betas, np.float64)
    gammas = _c(gammas, np.float64)
    p = betas.shape[0]
    ini = _c(ini, np.complex128)
    E = np.zeros(1)
    st = np.zeros(2 ** n, dtype=np.complex128) if want_state else None
    _chk(lib().qgo_qaoa_run(n, p, _p(betas), _p(gammas), len(terms), _p(terms.kind), _p(terms.q0), _p(terms.q1),
                            _p(terms.w), _p(ini), _p(E), _p(st)))
    return (float(E[0]), st) if want_state else float(E[0])


def maxcut_table(n, edges):
    edges = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
    t = np.zeros(2 ** n, dtype=np.int32)
    _chk(lib().qgo_maxcut_table(n, len(edges), _p(edges), _p(t)))
    return t


def entangle(n, state, kind, inverse=False):
    s = np.array(state, dtype=np.complex128, copy=True)
    _chk(lib().qgo_entangle(n, kind, int(bool(inverse)), _p(s)))
    return s


def num_threads():
    return lib().qgo_num_threads()

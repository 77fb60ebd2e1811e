"""Batched execution: many circuits in persistent launches, CUDA-graph captured.

Each job (one circuit + one parameter vector) runs a whole ``run`` or
``grad_run`` inside one cluster of the persistent kernel with the state in
shared memory (``qg_batch_launch``).  Jobs whose qubit count exceeds the
shared-memory limit fall back to the per-circuit sweep path, captured in the
same CUDA graph.  Circuits may differ in kind (McClean / QAOA), qubit count,
depth and observable.

    b = Batch(device="cuda", dtype="complex64")
    slots = [b.add(circuit) for circuit in circuits]      # McClean / Qaoa objects
    b.finalize()
    b.params[slot].copy_(...)                             # device parameters
    E, grads = b.grad()                                   # device tensors
"""
import ctypes

import numpy as np
import torch

from . import _lib, _native

# qg_batch_job (include/qgrad.h)
_JOB = np.dtype([("kind", "<i4"), ("n", "<i4"), ("layers", "<i4"), ("entangler", "<i4"), ("placement", "<i4"),
                 ("nterms", "<i4"), ("terms", "<u8"), ("axes", "<u8"), ("params", "<u8"), ("expec", "<u8"),
                 ("grad", "<u8"), ("cost_nterms", "<i4"), ("cost_maxabs", "<i4"), ("cost_w0", "<f8"),
                 ("cost", "<u8")])
assert _JOB.itemsize == 88
_TERM = np.dtype([("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("pad", "<i4"), ("w", "<f8")])
_COST = np.dtype([("b0", "<i4"), ("b1", "<i4"), ("c", "<i4"), ("pad", "<i4")])

_ENT = {"cnot": _lib.QG_ENT_CNOT_LADDER, "cz": _lib.QG_ENT_CZ_LADDER, None: _lib.QG_ENT_NONE,
        "none": _lib.QG_ENT_NONE}
_PLACE = {"before": _lib.QG_PLACE_BEFORE, "after": _lib.QG_PLACE_AFTER}

# largest qubit count held by one CTA / by a 2-CTA cluster
SINGLE_MAX = {_lib.QG_C64: 13, _lib.QG_C128: 12}
CLUSTER_MAX = {_lib.QG_C64: 14, _lib.QG_C128: 13}
MAX_COST = 511


def _dev_bytes(arr, device):
    a = np.ascontiguousarray(arr)
    t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).to(device)
    return t


class Batch:
    """A fixed list of jobs executed together; parameters live in ``params``."""

    def __init__(self, device=None, dtype="complex64", grad=True, use_graph=True, cluster_from=None):
        """cluster_from: smallest qubit count whose jobs are split over a
        2-CTA cluster (default: only jobs too large for one CTA);
        ``tuning.tune_batch`` picks it by timing."""
        self.device = _native.require_cuda(device)
        self.dtype = _native.dtype_code(dtype)
        self.want_grad = grad
        self.use_graph = use_graph
        self.cluster_from = SINGLE_MAX[self.dtype] + 1 if cluster_from is None else int(cluster_from)
        self._specs = []
        self._keep = []
        self._graph = None
        self.finalized = False

    # ------------------------------------------------------------ building
    def add(self, circuit, params=None):
        """Add a job for a McClean or Qaoa circuit object; returns its slot."""
        if self.finalized:
            raise RuntimeError("batch already finalized")
        from .circuit_logic import McClean, Qaoa

        if isinstance(circuit, McClean):
            kind = 0
            nparams = circuit.lnum * circuit.qnum
            p = circuit._angles() if params is None else params
        elif isinstance(circuit, Qaoa):
            kind = 1
            nparams = 2 * circuit.lnum
            p = params
        else:
            raise ValueError("expected a McClean or Qaoa circuit")
        self._specs.append({"circuit": circuit, "kind": kind, "nparams": nparams, "init": p})
        return len(self._specs) - 1

    def finalize(self):
        dev = self.device
        lib = _lib.load()
        total = sum(s["nparams"] for s in self._specs)
        B = len(self._specs)
        self.params_flat = torch.zeros(max(total, 1), dtype=torch.float64, device=dev)
        self.grads_flat = torch.zeros(max(total, 1), dtype=torch.float64, device=dev)
        self.expec = torch.zeros(max(B, 1), dtype=torch.float64, device=dev)
        self.params, self.grads = [], []
        off = 0
        for s in self._specs:
            s["off"] = off
            self.params.append(self.params_flat[off: off + s["nparams"]])
            self.grads.append(self.grads_flat[off: off + s["nparams"]])
            if s["init"] is not None:
                self.params[-1].copy_(torch.as_tensor(np.asarray(s["init"], dtype=np.float64)).reshape(-1))
            off += s["nparams"]
        self._structures = {}
        self._build_groups()
        self.finalized = True

    def refinalize(self, cluster_from):
        """Regroup the jobs with a new cluster split; parameters are kept."""
        if not self.finalized:
            self.cluster_from = int(cluster_from)
            return self.finalize()
        self.cluster_from = int(cluster_from)
        self._graph = None
        self._build_groups()

    def _build_groups(self):
        dev = self.device
        # shared structure buffers, one per distinct circuit object
        cache = self._structures
        small, clus, big = [], [], []
        single, cmax = SINGLE_MAX[self.dtype], CLUSTER_MAX[self.dtype]
        split = max(4, min(self.cluster_from, single + 1))
        for i, s in enumerate(self._specs):
            c = s["circuit"]
            key = id(c)
            if key not in cache:
                cache[key] = self._structure(c, s["kind"])
            st = cache[key]
            if c.qnum > cmax or st is None:
                big.append(i)
                continue
            job = np.zeros(1, dtype=_JOB)
            job["kind"] = s["kind"]
            job["n"] = c.qnum
            job["layers"] = c.lnum
            job["entangler"] = _ENT[c.entangler] if s["kind"] == 0 else 0
            job["placement"] = _PLACE[c.placement] if s["kind"] == 0 else 0
            job["nterms"] = st["nterms"]
            job["terms"] = st["terms"].data_ptr() if st["terms"] is not None else 0
            job["axes"] = st["axes"].data_ptr() if st["axes"] is not None else 0
            job["params"] = self.params[i].data_ptr()
            job["expec"] = self.expec[i:i + 1].data_ptr()
            job["grad"] = self.grads[i].data_ptr() if self.want_grad else 0
            job["cost_nterms"] = st["cost_nterms"]
            job["cost_maxabs"] = st["cost_maxabs"]
            job["cost_w0"] = st["cost_w0"]
            job["cost"] = st["cost"].data_ptr() if st["cost"] is not None else 0
            (small if c.qnum < split else clus).append((c.qnum, job))
        self._keep = list(cache.values())
        self._groups = []
        for cl, jobs in ((1, small), (2, clus)):
            if not jobs:
                continue
            arr = np.concatenate([j for _, j in jobs])
            maxq = max(q for q, _ in jobs)
            ws = torch.zeros(256, dtype=torch.uint8, device=dev)
            self._groups.append((cl, _dev_bytes(arr, dev), len(jobs), maxq, ws))
        self._big = big

    def _structure(self, c, kind):
        dev = self.device
        kindv, q0, q1, w = c.observable.terms
        terms = np.zeros(len(kindv), dtype=_TERM)
        terms["kind"], terms["q0"], terms["q1"], terms["w"] = kindv, q0, q1, w
        st = {"nterms": len(kindv), "terms": _dev_bytes(terms, dev) if len(kindv) else None, "axes": None,
              "cost": None, "cost_nterms": 0, "cost_maxabs": 0, "cost_w0": 1.0}
        if kind == 0:
            st["axes"] = torch.as_tensor(np.asarray(c.axes, dtype=np.int8).reshape(-1), device=dev)
        else:
            lib = _lib.load()
            out = np.zeros(600, dtype=_COST)
            nout, w0, maxabs = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_int(0)
            status = lib.qg_qaoa_cost_terms(c.qnum, len(kindv), kindv.ctypes.data_as(ctypes.c_void_p),
                                            q0.ctypes.data_as(ctypes.c_void_p), q1.ctypes.data_as(ctypes.c_void_p),
                                            w.ctypes.data_as(ctypes.c_void_p), 600,
                                            out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nout),
                                            ctypes.byref(w0), ctypes.byref(maxabs))
            if status != _lib.QG_OK or maxabs.value > MAX_COST:
                return None  # not representable in the batched kernel: sweep path
            st["cost"] = _dev_bytes(out[: nout.value], dev) if nout.value else None
            st["cost_nterms"], st["cost_maxabs"], st["cost_w0"] = nout.value, maxabs.value, w0.value
        return st

    # ------------------------------------------------------------ execution
    def _launch(self):
        lib = _lib.load()
        stream = _native.stream_handle(self.device)
        for cl, jobs, nj, maxq, ws in self._groups:
            _lib.check(lib.qg_batch_launch(self.dtype, _native.ptr(jobs), nj, maxq, cl, _native.ptr(ws), ws.numel(),
                                           stream))
        for i in self._big:
            s = self._specs[i]
            c = s["circuit"]
            nat = c.native()
            if self.want_grad:
                op = _lib.QG_OP_GRAD_UNCOMPUTE
                e, g = nat.grad(self.params[i], self.dtype, self.device, op,
                                out=(self.expec[i:i + 1], self.grads[i]))
            else:
                e, _ = nat.run(self.params[i], self.dtype, self.device)
                self.expec[i:i + 1].copy_(e)

    def _prepare_big(self):
        # allocate the sweep-path workspaces outside any graph capture
        for i in self._big:
            c = self._specs[i]["circuit"]
            op = _lib.QG_OP_GRAD_UNCOMPUTE if self.want_grad else _lib.QG_OP_RUN
            c.native().workspace(self.dtype, op, self.device)

    def execute(self):
        """Run every job once (graph replay after the first call)."""
        if not self.finalized:
            self.finalize()
        if not self.use_graph:
            self._launch()
            return self.expec, self.grads
        if self._graph is None:
            self._prepare_big()
            self._launch()  # warm-up outside capture (function attributes, lazy loading)
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._launch()
            self._graph = g
        self._graph.replay()
        return self.expec, self.grads

    def grad(self):
        if not self.want_grad:
            raise RuntimeError("batch built with grad=False")
        return self.execute()


def mcclean_batch(n, layers, axes, observable, nbatch, dtype="complex64", device=None, entangler="cnot",
                  placement="before", use_graph=True):
    """``nbatch`` parameter vectors of one McClean circuit (shared axes)."""
    from .circuit_logic import McClean

    c = McClean(n, observable, layers, axes=np.asarray(axes), angles=np.zeros((layers, n)), entangler=entangler,
                placement=placement, dtype=dtype, device=device)
    b = Batch(device=device, dtype=dtype, use_graph=use_graph)
    for _ in range(nbatch):
        b.add(c, params=None)
    b.finalize()
    return b

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
                 ("cost", "<u8"), ("term_expec", "<u8")])
assert _JOB.itemsize == 96
_TERM = np.dtype([("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("pad", "<i4"), ("w", "<f8")])
_COST = np.dtype([("b0", "<i4"), ("b1", "<i4"), ("c", "<i4"), ("pad", "<i4")])

_ENT = {"cnot": _lib.QG_ENT_CNOT_LADDER, "cz": _lib.QG_ENT_CZ_LADDER, None: _lib.QG_ENT_NONE,
        "none": _lib.QG_ENT_NONE, "cnot_periodic": _lib.QG_ENT_CNOT_LADDER_PERIODIC}
_PLACE = {"before": _lib.QG_PLACE_BEFORE, "after": _lib.QG_PLACE_AFTER}

# largest qubit count held by one CTA / by a 2-CTA cluster
SINGLE_MAX = {_lib.QG_C64: 13, _lib.QG_C128: 12}
CLUSTER_MAX = {_lib.QG_C64: 14, _lib.QG_C128: 13}
MAX_COST = 511


def _to_device(host, device):
    """Host array -> device tensor without synchronising the current stream:
    staged through pinned memory (whose block the host allocator keeps until
    the copy has run) and copied asynchronously in stream order.  A plain
    copy from pageable memory would wait for all earlier work on the stream."""
    return torch.from_numpy(host).pin_memory().to(device, non_blocking=True)


def _dev_bytes(arr, device):
    a = np.ascontiguousarray(arr)
    return _to_device(a.view(np.uint8).reshape(-1).copy(), device)


class Batch:
    """A fixed list of jobs executed together; parameters live in ``params``."""

    def __init__(self, device=None, dtype="complex64", grad=True, use_graph=True, cluster_from=None,
                 term_expectations=False):
        """cluster_from: smallest qubit count whose jobs are split over a
        2-CTA cluster (default: only jobs too large for one CTA);
        ``tuning.tune_batch`` picks it by timing.  term_expectations: also
        return <P_k> of every observable term of each job's final state
        (``term_expec[slot]``, for projector-shot estimates)."""
        self.device = _native.require_cuda(device)
        self.dtype = _native.dtype_code(dtype)
        self.want_grad = grad
        self.want_terms = term_expectations
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
        total = sum(s["nparams"] for s in self._specs)
        B = len(self._specs)
        # initial parameters packed on the host and copied in one transfer
        host = np.zeros(max(total, 1), dtype=np.float64)
        off = 0
        for s in self._specs:
            s["off"] = off
            if s["init"] is not None:
                init = s["init"]
                if isinstance(init, torch.Tensor):
                    init = init.detach().cpu().numpy()
                host[off: off + s["nparams"]] = np.asarray(init, dtype=np.float64).reshape(-1)
            off += s["nparams"]
        self.params_flat = _to_device(host, dev)
        # every output slot is written by the kernels (a 2-CTA job clears its
        # slots before adding to them), so no clearing is needed here
        self.grads_flat = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
        self.expec = torch.empty(max(B, 1), dtype=torch.float64, device=dev)
        self.params = [self.params_flat[s["off"]: s["off"] + s["nparams"]] for s in self._specs]
        self.grads = [self.grads_flat[s["off"]: s["off"] + s["nparams"]] for s in self._specs]
        toff = 0
        for s in self._specs:
            s["toff"] = toff
            toff += s["circuit"].observable.num_components if self.want_terms else 0
        self.term_expec_flat = torch.empty(max(toff, 1), dtype=torch.float64, device=dev)
        self.term_expec = [self.term_expec_flat[s["toff"]: s["toff"] + (s["circuit"].observable.num_components
                                                                         if self.want_terms else 0)]
                           for s in self._specs]
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
        # shared structure buffers, one per distinct circuit object, packed
        # into one device blob (one host-to-device copy for the batch)
        cache = self._structures
        self._upload_structures()
        single, cmax = SINGLE_MAX[self.dtype], CLUSTER_MAX[self.dtype]
        split = max(4, min(self.cluster_from, single + 1))
        # job tables filled column by column (one numpy assignment per field)
        cols = {k: [] for k in ("i", "kind", "n", "layers", "entangler", "placement", "nterms", "terms", "axes",
                                "cost_nterms", "cost_maxabs", "cost_w0", "cost", "periodic")}
        big = []
        for i, s in enumerate(self._specs):
            c = s["circuit"]
            st = cache[id(c)]
            # the periodic ladder targets the top qubit, which a 2-CTA job splits
            periodic = s["kind"] == 0 and c.entangler == "cnot_periodic"
            if c.qnum > cmax or st is None or (periodic and c.qnum > single):
                big.append(i)
                continue
            mc = s["kind"] == 0
            for k, v in (("i", i), ("kind", s["kind"]), ("n", c.qnum), ("layers", c.lnum),
                         ("entangler", _ENT[c.entangler] if mc else 0), ("placement", _PLACE[c.placement] if mc else 0),
                         ("nterms", st["nterms"]), ("terms", st["terms"]), ("axes", st["axes"]),
                         ("cost_nterms", st["cost_nterms"]), ("cost_maxabs", st["cost_maxabs"]),
                         ("cost_w0", st["cost_w0"]), ("cost", st["cost"]), ("periodic", periodic)):
                cols[k].append(v)
        idx = np.asarray(cols["i"], dtype=np.int64)
        qn = np.asarray(cols["n"], dtype=np.int64)
        offs = np.asarray([self._specs[i]["off"] for i in idx], dtype=np.uint64)
        toffs = np.asarray([self._specs[i]["toff"] for i in idx], dtype=np.uint64)
        pbase, gbase, ebase = self.params_flat.data_ptr(), self.grads_flat.data_ptr(), self.expec.data_ptr()
        tbase = self.term_expec_flat.data_ptr()
        self._groups = []
        per = np.asarray(cols["periodic"], dtype=bool)
        for cl, sel in ((1, (qn < split) | per), (2, (qn >= split) & ~per)):
            nj = int(sel.sum())
            if nj == 0:
                continue
            arr = np.zeros(nj, dtype=_JOB)
            for k in ("kind", "n", "layers", "entangler", "placement", "nterms", "terms", "axes", "cost_nterms",
                      "cost_maxabs", "cost_w0", "cost"):
                arr[k] = np.asarray(cols[k])[sel]
            arr["params"] = pbase + 8 * offs[sel]
            arr["expec"] = ebase + 8 * idx[sel].astype(np.uint64)
            arr["grad"] = gbase + 8 * offs[sel] if self.want_grad else 0
            arr["term_expec"] = tbase + 8 * toffs[sel] if self.want_terms else 0
            maxq = int(qn[sel].max())
            ws = torch.empty(256, dtype=torch.uint8, device=dev)  # job counter, cleared by qg_batch_launch
            self._groups.append((cl, _dev_bytes(arr, dev), nj, maxq, ws))
        self._big = big

    def _upload_structures(self):
        """Host arrays of every circuit not yet uploaded, packed 16-byte
        aligned into one buffer and copied to the device at once; the cache
        then holds device addresses."""
        pending, blobs, size, seen = [], [], 0, set()
        for s in self._specs:
            c = s["circuit"]
            if id(c) in self._structures or id(c) in seen:
                continue
            seen.add(id(c))
            st = self._structure(c, s["kind"])
            if st is None:
                self._structures[id(c)] = None  # runs on the sweep path
                continue
            offs = {}
            for key in ("terms", "axes", "cost"):
                a = st[key]
                if a is None:
                    continue
                b = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
                size = (size + 15) & ~15
                offs[key] = size
                blobs.append((size, b))
                size += b.size
            pending.append((c, st, offs))
        if not pending:
            return
        host = np.zeros(max(size, 16), dtype=np.uint8)
        for o, b in blobs:
            host[o:o + b.size] = b
        buf = _to_device(host, self.device)
        self._blobs = getattr(self, "_blobs", []) + [buf]
        base = buf.data_ptr()
        for c, st, offs in pending:
            for key in ("terms", "axes", "cost"):
                st[key] = base + offs[key] if key in offs else 0
            self._structures[id(c)] = st

    def _structure(self, c, kind):
        """Host-side structure arrays of one circuit (uploaded by the caller)."""
        kindv, q0, q1, w = c.observable.terms
        terms = np.zeros(len(kindv), dtype=_TERM)
        terms["kind"], terms["q0"], terms["q1"], terms["w"] = kindv, q0, q1, w
        st = {"nterms": len(kindv), "terms": terms if len(kindv) else None, "axes": None,
              "cost": None, "cost_nterms": 0, "cost_maxabs": 0, "cost_w0": 1.0}
        if kind == 0:
            st["axes"] = np.asarray(c.axes, dtype=np.int8).reshape(-1)
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
            st["cost"] = out[: nout.value].copy() if nout.value else None
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
                if self.want_terms and self.term_expec[i].numel():
                    _, st = nat.run(self.params[i], self.dtype, self.device, want_state=True)
                    nat.pauli_expectations_into(st, self.dtype, self.device, self.term_expec[i])
            else:
                e, st = nat.run(self.params[i], self.dtype, self.device, want_state=self.want_terms)
                self.expec[i:i + 1].copy_(e)
                if self.want_terms and self.term_expec[i].numel():
                    nat.pauli_expectations_into(st, self.dtype, self.device, self.term_expec[i])

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

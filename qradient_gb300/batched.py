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

# largest qubit count held by one CTA / a 2-CTA cluster / the batched kernel
# (4-CTA clusters above the pair limit)
SINGLE_MAX = {_lib.QG_C64: 13, _lib.QG_C128: 12}
PAIR_MAX = {_lib.QG_C64: 14, _lib.QG_C128: 13}
CLUSTER_MAX = {_lib.QG_C64: 15, _lib.QG_C128: 14}
MAX_COST = 511


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
        self._graph = None
        self._views = None
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
        specs = self._specs
        B = len(specs)
        off = toff = 0
        for sp in specs:
            sp["off"] = off
            off += sp["nparams"]
            nt = sp["circuit"].observable.num_components if self.want_terms else 0
            sp["toff"], sp["nterm"] = toff, nt
            toff += nt
        total = off
        # initial parameters packed on the host; they travel with the batch's
        # one host-to-device copy (_build_groups)
        host = np.zeros(max(total, 1), dtype=np.float64)
        for sp in specs:
            init = sp["init"]
            if init is not None:
                if isinstance(init, torch.Tensor):
                    init = init.detach().cpu().numpy()
                host[sp["off"]: sp["off"] + sp["nparams"]] = np.asarray(init, dtype=np.float64).reshape(-1)
        # outputs in one allocation: gradients | expectation values | term
        # expectations.  Every output slot is written by the kernels (a 2-CTA
        # job clears its slots before adding to them): no clearing is needed.
        ng, nb, ne = max(total, 1), max(B, 1), max(toff, 1)
        out = torch.empty(ng + nb + ne, dtype=torch.float64, device=dev)
        self.grads_flat, self.expec, self.term_expec_flat = out[:ng], out[ng:ng + nb], out[ng + nb:]
        self._views = None
        self._structures = {}
        self._build_groups(host)
        self.finalized = True

    # per-job views of the flat buffers, made on first use
    def _job_views(self):
        if self._views is None:
            sp = self._specs
            self._views = ([self.params_flat[s["off"]: s["off"] + s["nparams"]] for s in sp],
                           [self.grads_flat[s["off"]: s["off"] + s["nparams"]] for s in sp],
                           [self.term_expec_flat[s["toff"]: s["toff"] + s["nterm"]] for s in sp])
        return self._views

    @property
    def params(self):
        return self._job_views()[0]

    @property
    def grads(self):
        return self._job_views()[1]

    @property
    def term_expec(self):
        return self._job_views()[2]

    def refinalize(self, cluster_from):
        """Regroup the jobs with a new cluster split; parameters are kept."""
        if not self.finalized:
            self.cluster_from = int(cluster_from)
            return self.finalize()
        self.cluster_from = int(cluster_from)
        self._graph = None
        self._build_groups(None)

    def _build_groups(self, host_params):
        """Job tables per launch group.  Everything the batch uploads -- the
        initial parameters (host_params; None keeps the device ones), the
        structure arrays of circuits not uploaded yet, the job tables and
        the groups' job counters -- is packed into one host buffer and
        copied to one device allocation in a single asynchronous transfer."""
        dev = self.device
        cache = self._structures
        # structure arrays of new circuits, at offsets relative to their region
        pending, blobs, ssize, seen = [], [], 0, set()
        for sp in self._specs:
            c = sp["circuit"]
            if id(c) in cache or id(c) in seen:
                continue
            seen.add(id(c))
            st = self._structure(c, sp["kind"])
            if st is None:
                cache[id(c)] = None  # runs on the sweep path
                continue
            rel = {}
            for key in ("terms", "axes", "cost"):
                a = st[key]
                if a is None:
                    continue
                b = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
                ssize = (ssize + 15) & ~15
                rel[key] = ssize
                blobs.append((ssize, b))
                ssize += b.size
            pending.append((c, st, rel))
            cache[id(c)] = st
        single, cmax = SINGLE_MAX[self.dtype], CLUSTER_MAX[self.dtype]
        split = max(4, min(self.cluster_from, single + 1))
        # job rows, one list per field
        cols = {k: [] for k in ("i", "kind", "n", "layers", "entangler", "placement", "st", "periodic")}
        big = []
        for i, sp in enumerate(self._specs):
            c = sp["circuit"]
            st = cache[id(c)]
            # the periodic ladder targets the top qubit, which a 2-CTA job splits
            periodic = sp["kind"] == 0 and c.entangler == "cnot_periodic"
            if c.qnum > cmax or st is None or (periodic and c.qnum > single):
                big.append(i)
                continue
            mc = sp["kind"] == 0
            cols["i"].append(i)
            cols["kind"].append(sp["kind"])
            cols["n"].append(c.qnum)
            cols["layers"].append(c.lnum)
            cols["entangler"].append(_ENT[c.entangler] if mc else 0)
            cols["placement"].append(_PLACE[c.placement] if mc else 0)
            cols["st"].append(st)
            cols["periodic"].append(periodic)
        idx = np.asarray(cols["i"], dtype=np.int64)
        qn = np.asarray(cols["n"], dtype=np.int64)
        per = np.asarray(cols["periodic"], dtype=bool)
        groups = []
        pair = PAIR_MAX[self.dtype]
        for cl, sel in ((1, (qn < split) | per), (2, (qn >= split) & (qn <= pair) & ~per), (4, (qn > pair) & ~per)):
            nj = int(sel.sum()) if idx.size else 0
            if nj:
                groups.append((cl, sel, nj, int(qn[sel].max())))
        # layout of the upload: params | structures | job tables | job counters
        size = 0
        p_off = None
        if host_params is not None:
            p_off, size = 0, host_params.nbytes
        size = (size + 15) & ~15
        s_off = size
        size += ssize
        j_offs = []
        for cl, sel, nj, maxq in groups:
            size = (size + 15) & ~15
            j_offs.append(size)
            size += nj * _JOB.itemsize
        c_offs = []
        for _ in groups:
            size = (size + 255) & ~255
            c_offs.append(size)  # job counter, cleared by qg_batch_launch
            size += 256
        size = max((size + 15) & ~15, 16)
        blob = torch.empty(size, dtype=torch.uint8, device=dev)
        base = blob.data_ptr()
        host = np.zeros(size, dtype=np.uint8)
        if host_params is not None:
            host[p_off: p_off + host_params.nbytes] = host_params.view(np.uint8)
            self.params_flat = blob[p_off: p_off + host_params.nbytes].view(torch.float64)
        for o, b in blobs:
            host[s_off + o: s_off + o + b.size] = b
        for c, st, rel in pending:
            for key in ("terms", "axes", "cost"):
                st[key] = base + s_off + rel[key] if key in rel else 0
        offs = np.asarray([self._specs[i]["off"] for i in idx], dtype=np.uint64)
        toffs = np.asarray([self._specs[i]["toff"] for i in idx], dtype=np.uint64)
        pbase, gbase, ebase = self.params_flat.data_ptr(), self.grads_flat.data_ptr(), self.expec.data_ptr()
        tbase = self.term_expec_flat.data_ptr()
        sts = cols["st"]
        self._groups = []
        for (cl, sel, nj, maxq), jo, co in zip(groups, j_offs, c_offs):
            arr = np.zeros(nj, dtype=_JOB)
            for k in ("kind", "n", "layers", "entangler", "placement"):
                arr[k] = np.asarray(cols[k])[sel]
            ssel = [st for st, m in zip(sts, sel) if m]
            for k in ("nterms", "terms", "axes", "cost_nterms", "cost_maxabs", "cost_w0", "cost"):
                arr[k] = [st[k] for st in ssel]
            arr["params"] = pbase + 8 * offs[sel]
            arr["expec"] = ebase + 8 * idx[sel].astype(np.uint64)
            arr["grad"] = gbase + 8 * offs[sel] if self.want_grad else 0
            arr["term_expec"] = tbase + 8 * toffs[sel] if self.want_terms else 0
            host[jo: jo + arr.nbytes] = arr.view(np.uint8)
            self._groups.append((cl, blob[jo: jo + arr.nbytes], nj, maxq, blob[co: co + 256]))
        # one asynchronous copy in stream order, staged through pinned memory
        # (whose block the host allocator keeps until the copy has run)
        blob.copy_(torch.from_numpy(host).pin_memory(), non_blocking=True)
        self._blobs = getattr(self, "_blobs", []) + [blob]
        self._big = big

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
            status = lib.qg_qaoa_cost_terms(c.qnum, len(kindv), kindv.ctypes.data,
                                            q0.ctypes.data, q1.ctypes.data,
                                            w.ctypes.data, 600,
                                            out.ctypes.data, ctypes.byref(nout),
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

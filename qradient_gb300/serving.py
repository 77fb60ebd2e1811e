"""Continuous-batching request server for run / grad_run.

Requests (a McClean or Qaoa circuit, its parameters, 'run' or 'grad', a
dtype) arrive over time.  Each scheduling round:

1. completed work is retired: results copied to the host, latency recorded,
   its device memory returned to the admission budget;
2. queued requests are admitted in arrival order while their device
   footprint fits the budget (an adjoint request on the sweep path needs
   its workspace: the stored state history where that takes at most
   ``history_share`` of the budget -- the faster form, as ``grad_run``'s
   default picks it -- else the uncompute form's psi and lambda, doubled
   when the CNOT ladder needs ping-pong buffers; requests that fit the
   shared-memory kernel need only their parameters and outputs);
3. admitted small requests are packed into one batched persistent launch
   (``qg_batch_launch``) on the next of a few batch streams, each admitted
   large request gets its own stream running the sweep kernels.  Work from
   different rounds overlaps on the device: a round never waits for earlier
   launches, and host-to-device copies are asynchronous (pinned staging).

Results are identical to running the request alone (same kernels, same
reduction order); ``tests/test_gpu_serving.py`` checks this.

Failures stay per request: parameters of the wrong size or with non-finite
values are rejected by ``submit`` (``ValueError``, as the reference's
``Qaoa.__check_parameters`` raises for a wrong count); a launch or a
workspace allocation that raises fails the requests of that launch
(``Request.error`` holds the message, they go to ``failed``), returns their
footprint and stream, and leaves the server usable.  ``cancel(rid)``
withdraws a request that has not been admitted yet.
"""
import collections
import time

import numpy as np
import torch

from . import _lib, _native
from .batched import CLUSTER_MAX, PAIR_MAX, SINGLE_MAX, Batch


class Request:
    __slots__ = ("rid", "circuit", "params", "op", "dtype", "t_arrival", "t_done", "expec", "grad",
                 "footprint", "error", "_e", "_g", "_gop")

    def __init__(self, rid, circuit, params, op="grad", dtype="complex128", t_arrival=None):
        self.rid = rid
        self.circuit = circuit
        self.params = np.asarray(params, dtype=np.float64)
        if op not in ("grad", "run"):
            raise ValueError("op must be 'grad' or 'run'")
        self.op = op
        self.dtype = _native.dtype_code(dtype)
        self.t_arrival = time.perf_counter() if t_arrival is None else t_arrival
        self.t_done = None
        self.expec = None
        self.grad = None
        self.footprint = 0
        self.error = None
        self._e = self._g = None
        self._gop = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival

    @property
    def done(self):
        return self.t_done is not None

    @property
    def failed(self):
        return self.error is not None


def _state_bytes(n, dtype):
    return (2 ** n) * (16 if dtype == _lib.QG_C128 else 8)


class Server:
    """Admission by device-memory footprint, batched small requests, one
    stream per large request (up to ``streams`` concurrently)."""

    def __init__(self, device=None, hbm_budget=None, streams=8, max_batch=4096, batch_streams=8,
                 history_share=0.5):
        self.device = _native.require_cuda(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.5 * free)
        self.budget = int(hbm_budget)
        self.history_share = float(history_share)
        self.in_use = 0
        self.max_batch = max_batch
        self.queue = collections.deque()
        self.inflight = []
        self.finished = []
        self.failed = []
        self.rejected = []  # (schedule index, exception) of serve() entries that submit refused
        self.streams = [torch.cuda.Stream(self.device) for _ in range(streams)]
        self.stream_busy = [None] * streams
        # batches of consecutive rounds go to different streams: a round's
        # batch often has fewer jobs than the GPU has SMs, so batches overlap
        self.batch_streams = [torch.cuda.Stream(self.device) for _ in range(batch_streams)]
        self._next_batch_stream = 0
        self._rid = 0

    # ------------------------------------------------------------ interface
    def submit(self, circuit, params, op="grad", dtype="complex128", t_arrival=None):
        r = Request(self._rid, circuit, params, op, dtype, t_arrival)
        want = self._nparams(circuit)
        if r.params.size != want:
            raise ValueError("request needs %d parameters, got %d" % (want, r.params.size))
        if not np.all(np.isfinite(r.params)):
            raise ValueError("request parameters must be finite")
        self._rid += 1
        self._size(r)
        if r.footprint > self.budget:
            raise MemoryError("request needs %d bytes, above the server budget %d" % (r.footprint, self.budget))
        self.queue.append(r)
        return r

    def cancel(self, rid):
        """Withdraw a queued request; True if it was still waiting for
        admission (it then goes to ``failed`` with error 'cancelled'),
        False if it is already on the device or done."""
        for r in self.queue:
            if r.rid == rid:
                self.queue.remove(r)
                r.error = "cancelled"
                r.t_done = time.perf_counter()
                self.failed.append(r)
                return True
        return False

    @staticmethod
    def _nparams(circuit):
        kind = circuit.__class__.__name__
        if kind == "McClean":
            return circuit.lnum * circuit.qnum
        if kind == "Qaoa":
            return 2 * circuit.lnum
        raise ValueError("expected a McClean or Qaoa circuit")

    def _fail(self, reqs, exc):
        """Fail `reqs` after their launch raised: record the error, return
        their footprint, free their workspaces."""
        now = time.perf_counter()
        for r in reqs:
            r.error = "%s: %s" % (type(exc).__name__, exc)
            r.t_done = now
            r._e = r._g = None
            self.in_use -= r.footprint
            self.failed.append(r)
            if r.circuit._native is not None:
                r.circuit._native.release_workspaces()

    def _small(self, r):
        kind = r.circuit.__class__.__name__
        return r.circuit.qnum <= CLUSTER_MAX[r.dtype] and kind in ("McClean", "Qaoa")

    def _size(self, r):
        n = r.circuit.qnum
        if self._small(r):
            np_ = r.params.size
            r.footprint = 8 * (2 * np_ + 1) + 4096
        else:
            nat = r.circuit.native()
            if r.op == "grad":
                op = _lib.QG_OP_GRAD_HISTORY
                ws = nat.workspace_bytes(r.dtype, op)
                if ws > self.history_share * self.budget:
                    op = _lib.QG_OP_GRAD_UNCOMPUTE
                    ws = nat.workspace_bytes(r.dtype, op)
            else:
                op = _lib.QG_OP_RUN
                ws = nat.workspace_bytes(r.dtype, op)
            r._gop = op
            r.footprint = ws + 8 * (2 * r.params.size + 1)

    # ------------------------------------------------------------ scheduling
    def _retire(self):
        still = []
        for item in self.inflight:
            event, reqs, keep = item
            if not event.query():
                still.append(item)
                continue
            now = time.perf_counter()
            if isinstance(keep, Batch):
                # one device-to-host copy per output array of the batch
                E = keep.expec.cpu().numpy()
                G = keep.grads_flat.cpu().numpy() if keep.want_grad else None
            for k, r in enumerate(reqs):
                shape = (r.circuit.lnum, r.circuit.qnum) if r.circuit.__class__.__name__ == "McClean" else (
                    r.circuit.lnum, 2)
                if isinstance(keep, Batch):
                    r.expec = float(E[k])
                    if r.op == "grad":
                        off = keep._specs[k]["off"]
                        r.grad = G[off: off + keep._specs[k]["nparams"]].copy().reshape(shape)
                else:
                    r.expec = float(r._e.item())
                    if r.op == "grad":
                        r.grad = r._g.cpu().numpy().reshape(shape)
                r.t_done = now
                self.in_use -= r.footprint
                r._e = r._g = None
                self.finished.append(r)
            for i, s in enumerate(self.stream_busy):
                if s is item:
                    self.stream_busy[i] = None
                    # large request finished: give its workspace back
                    for r in reqs:
                        if r.circuit._native is not None:
                            r.circuit._native.release_workspaces()
        self.inflight = still

    def _admit(self):
        small, large = [], []
        free_streams = sum(1 for s in self.stream_busy if s is None)
        while self.queue:
            r = self.queue[0]
            if self.in_use + r.footprint > self.budget:
                break  # admission in arrival order: wait for memory to free up
            if not self._small(r) and len(large) >= free_streams:
                break  # no free stream for another large request yet
            self.queue.popleft()
            self.in_use += r.footprint
            (small if self._small(r) else large).append(r)
            if len(small) >= self.max_batch:
                break
        return small, large

    def _launch_small(self, reqs):
        # one batch per dtype and cluster size, each on the next batch stream:
        # the launches of a round overlap instead of queueing behind the
        # longest (4-CTA complex128 jobs, FP64-bound, run longest)
        by_key = collections.defaultdict(list)
        for r in reqs:
            n = r.circuit.qnum
            cls = 1 if n <= SINGLE_MAX[r.dtype] else 2 if n <= PAIR_MAX[r.dtype] else 4
            by_key[(r.dtype, cls)].append(r)
        for (dt, _), rs in by_key.items():
            st = self.batch_streams[self._next_batch_stream]
            self._next_batch_stream = (self._next_batch_stream + 1) % len(self.batch_streams)
            with torch.cuda.stream(st):
                try:
                    b = Batch(device=self.device, dtype=dt, grad=any(r.op == "grad" for r in rs), use_graph=False)
                    for r in rs:
                        b.add(r.circuit, params=r.params.reshape(-1))
                    b.finalize()
                    b.execute()
                    ev = torch.cuda.Event()
                    ev.record(st)
                except Exception as exc:  # the batch's requests fail, the server carries on
                    self._fail(rs, exc)
                    continue
            self.inflight.append((ev, rs, b))

    def _launch_large(self, r):
        idx = next(i for i, s in enumerate(self.stream_busy) if s is None)
        st = self.streams[idx]
        try:
            nat = r.circuit.native()
            with torch.cuda.stream(st):
                # asynchronous in stream order, staged through pinned memory
                params = torch.from_numpy(np.ascontiguousarray(r.params.reshape(-1))).pin_memory().to(
                    self.device, non_blocking=True)
                if r.op == "grad":
                    ws = nat.workspace(r.dtype, r._gop, self.device)
                    e, g = nat.grad(params, r.dtype, self.device, r._gop, workspace=ws)
                else:
                    ws = nat.workspace(r.dtype, _lib.QG_OP_RUN, self.device)
                    e, _ = nat.run(params, r.dtype, self.device, workspace=ws)
                    g = None
                r._e, r._g = e, g
                ev = torch.cuda.Event()
                ev.record(st)
        except Exception as exc:  # this request fails, its stream stays free
            self._fail([r], exc)
            return
        item = (ev, [r], (params, ws))
        self.stream_busy[idx] = item
        self.inflight.append(item)

    def step(self):
        """One scheduling round; returns the number of requests admitted."""
        self._retire()
        small, large = self._admit()
        if small:
            self._launch_small(small)
        for r in large:
            self._launch_large(r)
        return len(small) + len(large)

    def drain(self, timeout=600.0):
        """Step until every request has finished or failed; returns the finished ones."""
        t0 = time.perf_counter()
        while self.queue or self.inflight:
            if not self.step():
                time.sleep(0.0002)
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")
        return self.finished

    # ------------------------------------------------------------ workloads
    def serve(self, schedule):
        """Replay (t_offset, circuit, params, op, dtype) arrivals in real time
        and return the finished requests."""
        schedule = sorted(schedule, key=lambda s: s[0])
        t0 = time.perf_counter()
        i = 0
        while i < len(schedule) or self.queue or self.inflight:
            now = time.perf_counter() - t0
            while i < len(schedule) and schedule[i][0] <= now:
                off, c, p, op, dt = schedule[i]
                try:
                    self.submit(c, p, op, dt, t_arrival=t0 + off)
                except (ValueError, MemoryError) as exc:  # refused at the door; the stream goes on
                    self.rejected.append((i, exc))
                i += 1
            if not self.step():
                time.sleep(0.0002)
        return self.finished


def latency_stats(reqs):
    lat = np.array([r.latency for r in reqs if r.latency is not None]) * 1e3
    if lat.size == 0:
        return {}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": int(lat.size)}

"""Autotuner: picks the fusion depth and block shape of the kernels by timing.

Sweep path (one circuit per launch sequence): a sweep stages 2^t amplitudes
in shared memory and applies every rotation on those t bits in one pass, so
t is the fusion depth (fewer, larger passes against more shared memory per
CTA and fewer resident CTAs); the persistent grid is CTAs-per-SM x SMs; the
forward sweeps either load, compute and store one tile at a time or keep
the next tile's loads in flight in a second buffer.
``tune_circuit`` times grad_run (or run) for each candidate on a shortened
copy of the circuit (same qubits, axes of the first layers) and applies the
fastest to the circuit's handle (``qg_set_tuning``).

Batched path: jobs small enough for one CTA can instead be split over a
2-CTA cluster (half the state per CTA, the top qubit exchanged through
distributed shared memory), which halves the shared memory per CTA and the
per-job latency.  ``tune_batch`` times the batch's graph replay with the
split starting at different qubit counts and keeps the fastest.

Choices are cached per device, circuit shape and dtype in a JSON file
(``QG_TUNING_CACHE``, default ``_build/tuning.json`` beside the library), so
a shape is timed once per machine.
"""
import ctypes
import json
import os
import threading

import numpy as np
import torch

from . import _lib, _native

_LOCK = threading.Lock()
_MEM = {}


def cache_path():
    return os.environ.get("QG_TUNING_CACHE") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build",
                                                              "tuning.json")


def _load():
    p = cache_path()
    if p in _MEM:
        return _MEM[p]
    data = {}
    if os.path.exists(p):
        try:
            with open(p) as f:
                data = json.load(f)
        except (OSError, ValueError):
            data = {}
    _MEM[p] = data
    return data


def _store(key, value):
    with _LOCK:
        data = _load()
        data[key] = value
        p = cache_path()
        try:
            os.makedirs(os.path.dirname(p), exist_ok=True)
            tmp = p + ".tmp%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, p)
        except OSError:
            pass  # an unwritable cache only costs re-tuning


def _device_tag(device):
    return torch.cuda.get_device_name(device).replace(" ", "_")


def set_tuning(native, dtype, tile_bits=0, ctas_per_sm=0, flags=0):
    _lib.check(_lib.load().qg_set_tuning(native._h, dtype, int(tile_bits), int(ctas_per_sm), int(flags)))


def get_tuning(native, dtype):
    """Effective (tile_bits, ctas_per_sm, flags) of a handle."""
    t, c, f = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    _lib.check(_lib.load().qg_get_tuning(native._h, dtype, ctypes.byref(t), ctypes.byref(c), ctypes.byref(f)))
    return t.value, c.value, f.value


def sweep_candidates(dtype, n):
    """(tile_bits, ctas_per_sm, flags) triples: the default plan (tile_bits
    0: the library's per-sweep tile sizes), then three uniform fusion depths
    around the default, each at the occupancy-sized grid and at 1 CTA per
    SM, with plain and with pipelined (double-buffered) forward sweeps."""
    depths = (10, 11, 12) if dtype == _lib.QG_C128 else (11, 12, 13)
    lo = 5 if dtype == _lib.QG_C128 else 6
    depths = sorted({max(lo, min(t, n)) for t in depths})
    return [(0, 0, 0)] + [(t, c, f) for t in depths for c in (0, 1)
                          for f in (_lib.QG_TUNE_FWD_PLAIN, _lib.QG_TUNE_FWD_PIPELINED)]


def _time_ms(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _probe_circuit(circuit, layers):
    """A shortened native copy of the circuit for timing: same qubits,
    observable and entangler, the first `layers` layers."""
    from .circuit_logic import McClean

    if isinstance(circuit, McClean):
        L = min(circuit.lnum, layers)
        axes = np.asarray(circuit.axes)[:L]
        from .circuit_logic.mc_clean import _ENT, _PLACE

        nat = _native.NativeCircuit.mcclean(circuit.qnum, axes, circuit.observable.terms, _ENT[circuit.entangler],
                                            _PLACE[circuit.placement])
        return nat, L * circuit.qnum
    nat = _native.NativeCircuit.qaoa(circuit.qnum, min(circuit.lnum, layers), circuit.observable.terms)
    return nat, 2 * min(circuit.lnum, layers)


def _key(circuit, dtype, op, device):
    from .circuit_logic import McClean

    kind = "mcclean-%s-%s" % (circuit.entangler, circuit.placement) if isinstance(circuit, McClean) else "qaoa"
    return "sweep|%s|%s|n%d|%s|%s" % (_device_tag(device), kind, circuit.qnum,
                                      "c128" if dtype == _lib.QG_C128 else "c64", op)


def tune_circuit(circuit, op="grad", reps=3, layers=4, candidates=None, use_cache=True):
    """Time the candidates on a shortened copy of `circuit` and apply the
    fastest to its handle.  Returns {"tile_bits", "ctas_per_sm", "ms",
    "timings"}; the timings are per candidate, in ms per call of the copy."""
    dev = circuit._device()
    dtype = circuit._dtype_code
    key = _key(circuit, dtype, op, dev)
    if use_cache and candidates is None:
        hit = _load().get(key)
        if hit is not None:
            set_tuning(circuit.native(), dtype, hit["tile_bits"], hit["ctas_per_sm"], hit.get("flags", 0))
            return hit
    nat, nparams = _probe_circuit(circuit, layers)
    params = torch.rand(max(nparams, 1), dtype=torch.float64, device=dev)[:nparams] * 2 * np.pi
    e = torch.empty(1, dtype=torch.float64, device=dev)
    g = torch.empty(max(nparams, 1), dtype=torch.float64, device=dev)
    gop = _native.choose_grad_op(nat, dtype, dev, getattr(circuit, "grad_mode", "auto"))
    timings = []
    for t, c, f in candidates or sweep_candidates(dtype, circuit.qnum):
        set_tuning(nat, dtype, t, c, f)
        if op == "grad":
            ws = nat.workspace(dtype, gop, dev)
            fn = lambda: nat.grad(params, dtype, dev, gop, workspace=ws, out=(e, g))  # noqa: E731
        else:
            ws = nat.workspace(dtype, _lib.QG_OP_RUN, dev)
            fn = lambda: nat.run_into(params, dtype, dev, None, ws, e, None)  # noqa: E731
        timings.append({"tile_bits": t, "ctas_per_sm": c, "flags": f, "ms": _time_ms(fn, reps)})
        nat.release_workspaces()
    best = min(timings, key=lambda r: r["ms"])
    result = {"tile_bits": best["tile_bits"], "ctas_per_sm": best["ctas_per_sm"], "flags": best["flags"],
              "ms": best["ms"], "timings": timings}
    set_tuning(circuit.native(), dtype, best["tile_bits"], best["ctas_per_sm"], best["flags"])
    if use_cache and candidates is None:
        _store(key, result)
    return result


def tune_batch(batch, reps=3, use_cache=True):
    """Choose from which qubit count jobs run on 2-CTA clusters; re-finalizes
    the batch with the fastest choice.  Returns {"cluster_from", "ms",
    "timings"}."""
    from .batched import CLUSTER_MAX, SINGLE_MAX

    single, cmax = SINGLE_MAX[batch.dtype], CLUSTER_MAX[batch.dtype]
    qs = sorted({s["circuit"].qnum for s in batch._specs})
    key = "batch|%s|%s|%s" % (_device_tag(batch.device), "c128" if batch.dtype == _lib.QG_C128 else "c64",
                              ",".join("%d" % q for q in qs))
    choices = [single + 1] + [q for q in range(single, single - 3, -1) if q in qs and q >= 4]
    hit = _load().get(key) if use_cache else None
    if hit is not None and hit["cluster_from"] in choices:
        batch.refinalize(cluster_from=hit["cluster_from"])
        return hit
    timings = []
    for cf in choices:
        batch.refinalize(cluster_from=cf)
        timings.append({"cluster_from": cf, "ms": _time_ms(batch.execute, reps)})
    best = min(timings, key=lambda r: r["ms"])
    batch.refinalize(cluster_from=best["cluster_from"])
    result = {"cluster_from": best["cluster_from"], "ms": best["ms"], "timings": timings}
    if use_cache:
        _store(key, result)
    return result

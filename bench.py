"""Benchmark of the McClean adjoint grad_run on GB300.

Workload: McClean n=24 qubits, L=50 layers,
complex128, ZZ-chain observable sum_i Z_i Z_{i+1}, seeded random axes and
angles (numpy default_rng(24)), the reference's CNOT-ladder-before-rotations
layer.  A step is one full grad_run (E and all L*n gradients).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

value      circuits/s over the timed steps with inputs resident on the device
e2e        the same through the public API (McClean.grad_run) with host
           angles in (H2D) and host E + gradient out (D2H) every step
roofline   dominant kernel (the backward sweep): FP64-bound on GB300.  The
           achieved rate counts the FP64 instructions the kernel executes
           (ncu counts of the same workload, profiles/backward_sweep_traffic.json)
           against GB300's FP64 issue rate at the SM clock sampled during the
           timed region; the HBM view and the step-level T_roof / T_measured
           are reported beside it
cpu_baseline  the CPU oracle (C + OpenMP restatement of the reference's
           numpy algorithm) on the host cores, on a bounded sample
--impl reference  times that CPU restatement as the reference arm

The default run adds, measured in the same process after the headline:
  c64        the same circuit in complex64 (HBM-bound), with its HBM fraction
  cz_after   the same circuit with the CZ ladder after the rotations
  qaoa       QAOA MaxCut n=24 p=10 complex128
  large      McClean n=28 L=50 complex128 (its state history does not fit in
             HBM: the uncompute form of the adjoint sweep)
  batched    4096 parameter vectors of McClean n=14 L=30 complex64 in one
             CUDA-graph replay, against the plain per-call path
  batched_c128  the same circuit in complex128, 1024 vectors (4-CTA clusters)
  served     Poisson streams through the continuous-batching server (the
             n <= 14 share of the request population and the full n <= 26
             population), against the plain per-call path
(--headline-only skips them.)

Multi-GPU: replicas only (each rank runs its own circuit; no collective on
the data path), launched with torchrun; rank 0 prints the line.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--layers", type=int, default=50)
    ap.add_argument("--dtype", default="complex128", choices=["complex128", "complex64"])
    ap.add_argument("--entangler", default="cnot", choices=["cnot", "cz"])
    ap.add_argument("--placement", default="before", choices=["before", "after"])
    ap.add_argument("--grad-mode", default="auto", choices=["auto", "history", "uncompute"])
    ap.add_argument("--seed", type=int, default=24)
    ap.add_argument("--cpu-layers", type=int, default=10,
                    help="layers of the bounded CPU-baseline sample (same n, axes, angles)")
    ap.add_argument("--ref-layers", type=int, default=5,
                    help="reference arm: layers of the grad_run sample each step times (same n, axes, angles)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--workload", default="mcclean", choices=["mcclean", "batched", "qaoa", "serving"],
                    help="mcclean: one n=24 L=50 circuit (headline); batched: 4096 parameter vectors of an "
                         "n=14 L=30 circuit in one graph replay; qaoa: 3-regular MaxCut grad_run")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--autotune", action="store_true",
                    help="time the sweep-path variants for this circuit first (untimed) and use the fastest")
    ap.add_argument("--p", type=int, default=10, help="QAOA depth")
    ap.add_argument("--requests", type=int, default=120, help="serving: requests in the Poisson stream")
    ap.add_argument("--rate", type=float, default=0.0, help="serving: arrivals per second (0: saturate)")
    ap.add_argument("--max-qubits", type=int, default=26, help="serving: cap of the request qubit counts")
    ap.add_argument("--streams", type=int, default=8, help="serving: concurrent large requests (one stream each)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the nested c64 / cz_after / qaoa / batched / served measurements")
    return ap.parse_args()


def workload(n, L, seed):
    rng = np.random.default_rng(seed)
    axes = rng.integers(0, 3, (L, n))
    angles = rng.uniform(0, 2 * np.pi, (L, n))
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    return axes, angles, {"zz": zz}


def algorithmic(n, L, dtype):
    """Per-circuit bytes and FP64/FP32 flops of the compulsory model:
    B = S (6L + 4) (forward R+W per layer, observable, backward R+W of psi and
    lambda per layer), F = 2^n (6 n (L+1) + 12 n L + 4 n L + 6)."""
    S = (2 ** n) * (16 if dtype == "complex128" else 8)
    B = S * (6 * L + 4)
    F = (2 ** n) * (6 * n * (L + 1) + 12 * n * L + 4 * n * L + 6)
    return B, F


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_value(world, ms_per_step):
    """Whole-job circuits/s of `world` replicas, each one circuit per step,
    timed by the slowest rank."""
    return world * 1e3 / ms_per_step


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# GB300 FP64: 2 FMA lanes per SM per clock (a warp's DFMA holds the pipe for
# 16 cycles), 152 SMs; 4 flops per SM per clock counting an FMA as 2
GB300_SMS = 152
FP64_FLOPS_PER_SM_CLK = 4


def cpu_info():
    """CPU model, logical cores and OMP_NUM_THREADS of this host."""
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.startswith("model name"):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu_model": model, "nproc": os.cpu_count(), "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}


def cpu_sample(n, axes, angles, layers):
    """The CPU oracle's grad_run of the first `layers` layers of the circuit:
    returns the seconds it took."""
    from oracle import oracle as O

    t = O.Terms(np.full(n - 1, 3), np.arange(n - 1), np.arange(1, n), np.ones(n - 1))
    t0 = time.perf_counter()
    O.mcclean_grad(n, axes[:layers], angles[:layers], t)
    return time.perf_counter() - t0


def cpu_baseline(n, L, axes, angles, layers):
    """The CPU oracle (C + OpenMP restatement of the reference algorithm) on
    the first `layers` layers of the same circuit; scaled to circuits/s of
    the full L-layer circuit."""
    from oracle import oracle as O

    Ls = min(L, layers)
    dt = cpu_sample(n, axes, angles, Ls)
    d = {"value": Ls / (dt * L), "unit": "circuits/s", "cores": O.num_threads(), "kind": "port",
         "sample": "oracle/qg_oracle.c grad_run of the first %d of %d layers (n=%d), %.1f s, scaled by L/%d" %
                   (Ls, L, n, dt, Ls)}
    d.update(cpu_info())
    return d


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's grad_run on
    this host's cores.  Each step is a bounded sample, the grad_run of the
    first --cpu-layers layers of the headline circuit, and `value` scales it
    to circuits/s of the full circuit; one full L-layer grad_run is timed
    once as well (full_circuit_s), which checks that scaling.  --ref-layers
    sets the sample (5 of the 50 layers by default)."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    axes, angles, _ = workload(args.n, args.layers, args.seed)
    from oracle import oracle as O

    O.build()
    Ls = min(args.layers, args.ref_layers)
    for _ in range(args.warmup):
        cpu_sample(args.n, axes, angles, Ls)
    times = [cpu_sample(args.n, axes, angles, Ls) for _ in range(args.steps)]
    t = float(np.mean(times))
    value = Ls / (t * args.layers)
    full_s = cpu_sample(args.n, axes, angles, args.layers)
    cb = {"value": value, "unit": "circuits/s", "cores": O.num_threads(), "kind": "port",
          "sample": "each step: oracle/qg_oracle.c grad_run of the first %d of the %d layers (n=%d), %.2f s mean; "
                    "value = %d / (step time x %d)" % (Ls, args.layers, args.n, t, Ls, args.layers),
          "full_circuit_s": full_s, "full_circuit_value": 1.0 / full_s,
          "scaling_check": (1.0 / full_s) / value}
    cb.update(cpu_info())
    line = {"impl": "reference", "metric": "grad_run circuits/s", "value": value, "unit": "circuits/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "step_is_sample_of": "%d of %d layers" % (Ls, args.layers),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded axes/angles)",
            "config": config_of(args),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "circuits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config_of(args):
    S = (2 ** args.n) * (16 if args.dtype == "complex128" else 8)
    return {"workload": "McClean grad_run n=%d L=%d %s, ZZ-chain observable, %s ladder %s rotations" %
                        (args.n, args.layers, args.dtype, args.entangler, args.placement),
            "n": args.n, "layers": args.layers, "entangler": args.entangler, "placement": args.placement,
            "grad_mode": args.grad_mode, "seed": args.seed,
            "l2": ("inputs larger than L2 (state %d MiB > 129 MB)" if S > 129e6 else
                   "state of %d MiB fits in L2") % (S >> 20),
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def _events(dev):
    import torch

    return (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
            torch.cuda.current_stream(dev))


def measure_mcclean(n, L, seed, dtype, entangler, placement, steps, warmup, dev, min_warmup=3):
    """grad_run circuits/s of one McClean chain circuit (device-resident
    angles), with its step-level HBM fraction of the compulsory bytes."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300 import _lib, _native

    axes, angles, obs = workload(n, L, seed)
    c = McClean(n, obs, L, axes=axes, angles=angles, dtype=dtype, entangler=entangler, placement=placement,
                device=dev)
    a = torch.as_tensor(angles, dtype=torch.float64, device=dev).reshape(-1)
    out = (torch.empty(1, dtype=torch.float64, device=dev), torch.empty(n * L, dtype=torch.float64, device=dev))
    for _ in range(max(warmup, min_warmup)):
        c.grad_run_tensors(a, out=out)
    torch.cuda.synchronize()
    e0, e1, st = _events(dev)
    e0.record(st)
    for _ in range(steps):
        c.grad_run_tensors(a, out=out)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    B, _ = algorithmic(n, L, dtype)
    hbm = measured_peaks().get("hbm_gbs", 6800.0)
    res = {"workload": "McClean grad_run n=%d L=%d %s, %s ladder %s rotations" % (n, L, dtype, entangler, placement),
           "value": 1e3 / ms, "unit": "circuits/s", "ms_per_step": ms, "steps": steps,
           "hbm_gbs_algorithmic": B / ms * 1e-6, "hbm_frac_step": B / ms * 1e-6 / hbm,
           "hbm_peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    op = _native.choose_grad_op(c.native(), c._dtype_code, dev, c.grad_mode)
    res["grad_mode"] = "history" if op == _lib.QG_OP_GRAD_HISTORY else "uncompute"
    c._native.release_workspaces()
    return res


def measure_qaoa(n, p, seed, dtype, steps, warmup, dev, grad_mode="auto"):
    """QAOA MaxCut grad_run circuits/s on a seeded random 3-regular graph."""
    import torch

    from qradient_gb300 import Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    edges = random_regular_edges(3, n, seed)
    rng = np.random.default_rng(seed)
    betas, gammas = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    q = Qaoa(n, MaxCut(n, edge_set=edges).to_observable(), p, dtype=dtype, device=dev, grad_mode=grad_mode)
    params = torch.tensor(np.stack([betas, gammas], 1).reshape(-1), device=dev)
    nat = q.native()
    op = q._grad_op(nat)
    for _ in range(max(warmup, 3)):
        nat.grad(params, q._dtype_code, dev, op)
    torch.cuda.synchronize()
    e0, e1, st = _events(dev)
    e0.record(st)
    for _ in range(steps):
        nat.grad(params, q._dtype_code, dev, op)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    S = (2 ** n) * (16 if dtype == "complex128" else 8)
    hbm = measured_peaks().get("hbm_gbs", 6800.0)
    res = {"workload": "QAOA MaxCut grad_run n=%d p=%d %s, %d edges (seeded random 3-regular)" %
                       (n, p, dtype, len(edges)),
           "value": 1e3 / ms, "unit": "circuits/s", "ms_per_step": ms, "steps": steps,
           "hbm_gbs_algorithmic": S * (6 * p + 4) / ms * 1e-6, "hbm_frac_step": S * (6 * p + 4) / ms * 1e-6 / hbm,
           "_q": q, "_betas": betas, "_gammas": gammas, "_edges": edges}
    return res


def measure_batched(n, L, B, dtype, steps, warmup, seed, dev, e2e=True):
    """B parameter vectors (uniform [0, 2 pi)) of one McClean circuit with
    shared random axes in one CUDA-graph replay of the persistent
    shared-memory kernel, against the plain per-call GPU path (one grad_run
    at a time through the sweep kernels, device-resident parameters)."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.batched import mcclean_batch

    rng = np.random.default_rng(seed)
    axes = rng.integers(0, 3, (L, n))
    zz = np.full((n, n), None)
    for i in range(n - 1):
        zz[i, i + 1] = 1.0
    b = mcclean_batch(n, L, axes, {"zz": zz}, B, dtype=dtype, device=dev)
    P = torch.tensor(rng.uniform(0, 2 * np.pi, (B, L * n)), dtype=torch.float64, device=dev)
    b.params_flat.copy_(P.reshape(-1))
    for _ in range(max(warmup, 3)):
        b.grad()
    torch.cuda.synchronize()
    e0, e1, st = _events(dev)
    e0.record(st)
    for _ in range(steps):
        b.grad()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    value = B * 1e3 / ms
    c = McClean(n, {"zz": zz}, L, axes=axes, angles=P[0].reshape(L, n).cpu().numpy(), dtype=dtype, device=dev)
    out = (torch.empty(1, dtype=torch.float64, device=dev), torch.empty(n * L, dtype=torch.float64, device=dev))
    for _ in range(3):
        c.grad_run_tensors(angles=P[0], out=out)
    torch.cuda.synchronize()
    nplain = min(B, 64)
    e0.record(st)
    for k in range(nplain):
        c.grad_run_tensors(angles=P[k], out=out)
    e1.record(st)
    torch.cuda.synchronize()
    plain = nplain * 1e3 / e0.elapsed_time(e1)
    res = {"workload": "McClean grad_run n=%d L=%d %s, %d parameter vectors, shared axes, one CUDA-graph replay of "
                       "the persistent shared-memory kernel" % (n, L, dtype, B),
           "value": value, "unit": "circuits/s", "ms_per_step": ms, "steps": steps,
           "plain_per_call_circuits_s": plain, "speedup_vs_plain": value / plain,
           "flops_per_circuit": 2 ** n * (6 * n * (L + 1) + 16 * n * L + 6)}
    if e2e:
        # host parameters in, host E + gradients out, per replay
        Ph = P.cpu().pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            b.params_flat.copy_(Ph.reshape(-1), non_blocking=True)
            E, _ = b.grad()
            E.cpu()
            b.grads_flat.cpu()
        torch.cuda.synchronize()
        res["e2e"] = {"value": B * steps / (time.perf_counter() - t0), "unit": "circuits/s",
                      "h2d_bytes_per_step": B * L * n * 8, "d2h_bytes_per_step": B * (L * n + 1) * 8}
    return res


def serving_mix(seed, count, max_qubits=26):
    """Mixed request population: 60% McClean n ~ U{8..26}, L ~ U{5..60}; 40%
    QAOA 3-regular MaxCut n ~ U{10..24} (even), p ~ U{1..6}; dtype per
    request.  max_qubits caps both qubit ranges (the small-circuit share of
    the same population)."""
    from qradient_gb300 import McClean, Qaoa
    from qradient_gb300.optimization_problems import MaxCut, random_regular_edges

    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        dtype = "complex128" if rng.random() < 0.5 else "complex64"
        op = "grad" if rng.random() < 0.7 else "run"
        if rng.random() < 0.6:
            n = int(rng.integers(8, min(26, max_qubits) + 1))
            L = int(rng.integers(5, 61))
            zz = np.full((n, n), None)
            for i in range(n - 1):
                zz[i, i + 1] = 1.0
            c = McClean(n, {"zz": zz}, L, axes=rng.integers(0, 3, (L, n)), angles=np.zeros((L, n)), dtype=dtype,
                        grad_mode="uncompute")
            prm = rng.uniform(0, 2 * np.pi, (L, n))
        else:
            n = int(rng.integers(5, min(12, max_qubits // 2) + 1)) * 2
            p = int(rng.integers(1, 7))
            c = Qaoa(n, MaxCut(n, edge_set=random_regular_edges(3, n, seed * 1000 + k)).to_observable(), p,
                     dtype=dtype, grad_mode="uncompute")
            prm = np.stack([rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)], axis=1)
        reqs.append((c, prm, op, dtype))
    return reqs


def measure_served(seed, count, max_qubits, streams, dev, rate=0.0):
    """A Poisson stream of the mixed request population through the
    continuous-batching server, against the plain per-call path (each
    request alone through the public API, one after the other)."""
    import torch

    from qradient_gb300 import McClean
    from qradient_gb300.serving import Server, latency_stats

    reqs = serving_mix(seed, count, max_qubits)

    def alone(c, prm, op):
        if isinstance(c, McClean):
            c.angles = prm
            return c.grad_run() if op == "grad" else c.run_expec_val()
        return c.grad_run(prm[:, 0], prm[:, 1]) if op == "grad" else c.run_expec_val(prm[:, 0], prm[:, 1])

    for c, prm, op, dt in reqs[:4]:
        alone(c, prm, op)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c, prm, op, dt in reqs:
        alone(c, prm, op)
        if c._native is not None:
            c._native.release_workspaces()
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain = len(reqs) / plain_s
    # saturating arrival rate: at 30x the plain rate both populations queue
    # (the n <= 14 stream's capacity is 16-19k circuits/s, about 17x plain;
    # at 10x its arrivals, not the server, would set the throughput)
    rate = rate if rate > 0 else 30.0 * plain
    rng = np.random.default_rng(seed + 7)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    srv = Server(device=dev, streams=streams)
    # warm-up round (kernel attributes, lazy module loading)
    srv.serve([(0.0, c, prm, op, dt) for c, prm, op, dt in reqs[:4]])
    srv.finished.clear()
    t0 = time.perf_counter()
    done = srv.serve([(float(a), c, prm, op, dt) for a, (c, prm, op, dt) in zip(arrivals, reqs)])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    st = latency_stats(done)
    value = len(done) / wall
    return {"workload": "mixed request stream: 60%% McClean n~U{8..%d} L~U{5..60}, 40%% QAOA 3-regular "
                        "n~U{10..%d} p~U{1..6}, 70%% grad_run / 30%% run, dtype per request; %d requests, Poisson "
                        "rate %.1f/s" % (min(26, max_qubits), 2 * min(12, max_qubits // 2), len(reqs), rate),
            "value": value, "unit": "circuits/s", "wall_s": wall, "requests": len(done), "latency": st,
            "plain_per_call_circuits_s": plain, "speedup_vs_plain": value / plain}


def _public(d):
    return {k: v for k, v in d.items() if not k.startswith("_")}


def run_batched(args):
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    clocks = ClockSampler(local)
    clocks.start()
    r = measure_batched(args.n, args.layers, args.batch, args.dtype, args.steps, args.warmup, args.seed + rank, dev,
                        e2e=not args.no_e2e)
    clk = clocks.stop()
    line = {"metric": "batched grad_run circuits/s", "value": r["value"] * world, "unit": "circuits/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.dtype == "complex64" else "f64", "data": "synthetic (seeded axes/angles)",
            "config": {"workload": r["workload"],
                       "l2": "states live in shared memory; the parameter block streams once"},
            "plain_per_call_circuits_s": r["plain_per_call_circuits_s"], "speedup_vs_plain": r["speedup_vs_plain"],
            "gpu_launches": args.steps, "clocks": clk}
    if "e2e" in r:
        line["e2e"] = r["e2e"]
    if rank == 0:
        print(json.dumps(line))


def run_qaoa(args):
    """QAOA MaxCut grad_run on a seeded random 3-regular graph (n=24, p=10
    by default, complex128), plus 100 Philox shots from the final state."""
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    clocks = ClockSampler(local)
    clocks.start()
    r = measure_qaoa(args.n, args.p, args.seed + rank, args.dtype, args.steps, args.warmup, dev, args.grad_mode)
    clk = clocks.stop()
    q, betas, gammas = r["_q"], r["_betas"], r["_gammas"]
    q.run_expec_val(betas, gammas)
    shots = q.sample(100, seed=args.seed).cpu().numpy()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q.grad_run(betas, gammas)
    e2e = args.steps / (time.perf_counter() - t0)
    S = (2 ** args.n) * (16 if args.dtype == "complex128" else 8)
    line = {"metric": "QAOA grad_run circuits/s", "value": r["value"] * world, "unit": "circuits/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.dtype == "complex128" else "f32",
            "data": "synthetic (seeded random 3-regular graph, beta/gamma uniform [0, pi))",
            "config": {"workload": r["workload"], "l2": "inputs larger than L2" if S > 129e6 else "state fits in L2"},
            "hbm_gbs_algorithmic": r["hbm_gbs_algorithmic"],
            "shots_mean_cost": float(np.mean(q.classical_ham()[shots])) if args.n <= 26 else None,
            "e2e": {"value": e2e, "unit": "circuits/s", "h2d_bytes_per_step": 2 * args.p * 8,
                    "d2h_bytes_per_step": (2 * args.p + 1) * 8},
            "clocks": clk}
    if rank == 0:
        print(json.dumps(line))


def run_serving(args):
    """Poisson stream of a mixed McClean / QAOA request population through the continuous-batching
    server; compared with the plain per-call GPU path on the same requests."""
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    clocks = ClockSampler(local)
    clocks.start()
    r = measure_served(args.seed + rank, args.requests, args.max_qubits, args.streams, dev, args.rate)
    clk = clocks.stop()
    line = {"metric": "served circuits/s (run + grad_run mix)", "value": r["value"] * world, "unit": "circuits/s",
            "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": r["wall_s"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed f64/f32", "data": "synthetic Poisson stream",
            "config": {"workload": r["workload"]},
            "latency": r["latency"], "plain_per_call_circuits_s": r["plain_per_call_circuits_s"],
            "speedup_vs_plain": r["speedup_vs_plain"],
            "e2e": {"value": r["value"] * world, "unit": "circuits/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None}, "clocks": clk}
    if rank == 0:
        print(json.dumps(line))


def executed_fp64(dtype, n, L, seed):
    """Executed FP64 work of the headline workload per grad_run, from the ncu
    capture summarised in profiles/backward_sweep_traffic.json: per kernel
    class, the DFMA / DMUL / DADD thread instructions of every launch of one
    grad_run (flops = 2 DFMA + DMUL + DADD), and the DRAM bytes per backward
    launch.  None when the capture does not match the workload."""
    tpath = os.path.join(ROOT, "profiles", "backward_sweep_traffic.json")
    try:
        prof = json.load(open(tpath)).get(dtype) or {}
    except (OSError, ValueError):
        return None
    if prof.get("n") != n:
        return None
    ex = prof.get("executed_fp64") or {}
    if ex.get("layers") != L or ex.get("seed") != seed:
        ex = {}
    return {"traffic": prof.get("dram_bytes_per_launch"), "pipe_busy": prof.get("fp64_pipe_busy_ncu"),
            "executed": ex}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "qaoa":
        return run_qaoa(args)
    if args.workload == "serving":
        return run_serving(args)
    import torch

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from qradient_gb300 import McClean, _lib

    lib = _lib.load()
    axes, angles, obs = workload(args.n, args.layers, args.seed + rank)
    circ = McClean(args.n, obs, args.layers, axes=axes, angles=angles, dtype=args.dtype,
                   entangler=args.entangler, placement=args.placement, grad_mode=args.grad_mode, device=dev)
    angles_dev = torch.as_tensor(angles, dtype=torch.float64, device=dev).reshape(-1)
    out = (torch.empty(1, dtype=torch.float64, device=dev),
           torch.empty(args.n * args.layers, dtype=torch.float64, device=dev))

    tuned = None
    if args.autotune:
        from qradient_gb300 import tuning

        tuned = tuning.tune_circuit(circ, op="grad", use_cache=False)

    def step():
        circ.grad_run_tensors(angles_dev, out=out)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    import ctypes

    phys = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    idx = phys.split(",")[local] if phys else str(local)
    clocks = ClockSampler(idx)
    clocks.start()
    stream = torch.cuda.current_stream(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    # per-kernel durations from a second pass of the same steps with an event
    # pair around every launch (kept out of the timed region above: the
    # events cost a little per launch)
    lib.qg_profile_enable(1)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_prof = e0.elapsed_time(e1)
    kinfo = {}
    for cls, name in ((0, "forward_sweep"), (1, "backward_sweep"), (2, "observable")):
        tot = ctypes.c_double(0.0)
        cnt = ctypes.c_int(0)
        _lib.check(lib.qg_profile_collect(cls, ctypes.byref(tot), ctypes.byref(cnt)))
        kinfo[name] = (tot.value, cnt.value)
    lib.qg_profile_enable(0)
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = replica_value(world, ms_per_step)

    # end to end through the public API: host angles in, host E + grad out
    e2e_s = float("nan")
    if not args.no_e2e:
        for _ in range(2):
            circ.grad_run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            circ.angles = angles
            E, g = circ.grad_run()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    circ._native.release_workspaces()

    B, F = algorithmic(args.n, args.layers, args.dtype)
    bwd_ms, bwd_n = kinfo["backward_sweep"]
    fwd_ms, fwd_n = kinfo["forward_sweep"]
    S = (2 ** args.n) * (16 if args.dtype == "complex128" else 8)
    # algorithmic bytes of one backward launch: psi and lambda read, lambda written
    per_launch_bytes = 3 * S
    bwd_per_step = max(bwd_n / args.steps, 1)
    bwd_avg_s = bwd_ms / max(bwd_n, 1) * 1e-3
    achieved_gbs = per_launch_bytes / bwd_avg_s * 1e-9 if bwd_n else None
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    prof = executed_fp64(args.dtype, args.n, args.layers, args.seed) or {}
    ex = prof.get("executed") or {}
    share = {k: v[0] / ms_prof for k, v in kinfo.items()}
    if args.dtype == "complex128":
        sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
        fp64_peak = FP64_FLOPS_PER_SM_CLK * GB300_SMS * sm_mhz * 1e6 * 1e-12  # TFLOP/s
        bex = ex.get("backward") or {}
        fex = ex.get("forward") or {}
        achieved = None
        if bex.get("flops") and bwd_n:
            achieved = bex["flops"] / bex["launches"] / bwd_avg_s * 1e-12
        # step level: the binding roof of the whole grad_run
        step_flops = (bex.get("flops") or 0) + (fex.get("flops") or 0) + ((ex.get("other") or {}).get("flops") or 0)
        t_roof_ms = max(B / (hbm_peak * 1e9), step_flops / (fp64_peak * 1e12)) * 1e3 if step_flops else None
        roof = {"bound": "fp64", "kernel": "sweep_bwd_kernel<double,history,11>", "achieved": achieved,
                "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak if achieved else None,
                "traffic": prof.get("traffic"),
                "peak_source": "GB300 FP64 issue rate: 2 DFMA lanes per SM per clock (4 flops) x 152 SMs x the "
                               "median SM clock sampled during the timed region (%.0f MHz)" % sm_mhz,
                "achieved_source": "FP64 flops the backward launches execute (2 DFMA + DMUL + DADD thread "
                                   "instructions, ncu, every backward launch of one grad_run of this workload: "
                                   "profiles/backward_sweep_traffic.json) / their mean duration (CUDA events "
                                   "around every launch on the launching stream)",
                "fp64_pipe_busy_ncu": prof.get("pipe_busy"),
                # the credited algorithmic count (6 flops per rotation as the
                # reference's gate formula writes it, 4 per reduction, per
                # amplitude) at the same duration, for reference
                "algorithmic_rate_tflops": (2 ** args.n) * args.n * (4 + 6) * args.layers / bwd_per_step /
                                           bwd_avg_s * 1e-12 if bwd_n else None,
                "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                        "frac": achieved_gbs / hbm_peak if achieved_gbs else None,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
                "step": {"t_roof_ms": t_roof_ms, "t_measured_ms": ms_per_step,
                         "frac": t_roof_ms / ms_per_step if t_roof_ms else None,
                         "executed_fp64_flops": step_flops or None, "algorithmic_bytes": B},
                "launch_ms_avg": bwd_avg_s * 1e3, "launches": bwd_n, "kernel_share": share}
    else:
        roof = {"bound": "hbm", "kernel": "sweep_bwd_kernel<float,history,12>", "achieved": achieved_gbs,
                "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak if achieved_gbs else None,
                "traffic": prof.get("traffic"), "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                "step": {"t_roof_ms": B / (hbm_peak * 1e9) * 1e3, "t_measured_ms": ms_per_step,
                         "frac": B / (hbm_peak * 1e9) * 1e3 / ms_per_step, "algorithmic_bytes": B},
                "launch_ms_avg": bwd_avg_s * 1e3, "launches": bwd_n, "kernel_share": share}

    launches_per_step = (fwd_n + bwd_n + kinfo["observable"][1]) / args.steps + 1  # + the finalize kernel
    line = {
        "metric": "grad_run circuits/s", "value": value, "unit": "circuits/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.dtype == "complex128" else "f32",
        "data": "synthetic (seeded axes/angles)", "config": config_of(args),
        "hbm_gbs_algorithmic": B * value * 1e-9,
        "e2e": {"value": world / e2e_s, "unit": "circuits/s", "h2d_bytes_per_step": angles.size * 8,
                "d2h_bytes_per_step": (angles.size + 1) * 8},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "roofline": roof,
        "clocks": clk,
    }
    from qradient_gb300 import tuning as _tuning

    t_eff, c_eff, f_eff = _tuning.get_tuning(circ.native(), circ._dtype_code)
    line["config"]["tile_bits"] = t_eff
    line["config"]["ctas_per_sm"] = c_eff
    line["config"]["forward_sweeps"] = "pipelined" if f_eff == _lib.QG_TUNE_FWD_PIPELINED else "plain"
    if tuned is not None:
        line["config"]["autotune"] = {"chosen": [tuned["tile_bits"], tuned["ctas_per_sm"], tuned["flags"]],
                                      "ms_by_candidate": {"%d/%d/%d" % (r["tile_bits"], r["ctas_per_sm"], r["flags"]):
                                                          r["ms"] for r in tuned["timings"]}}
    if rank == 0 and not args.headline_only and args.n == 24 and args.layers == 50:
        # the rest of the metric, measured in this process after the headline
        t0 = time.perf_counter()
        extra_clk = ClockSampler(idx)
        extra_clk.start()
        other = "complex64" if args.dtype == "complex128" else "complex128"
        line["c64" if other == "complex64" else "c128"] = measure_mcclean(
            args.n, args.layers, args.seed, other, args.entangler, args.placement, 5, 3, dev)
        line["cz_after"] = measure_mcclean(args.n, args.layers, args.seed, args.dtype, "cz", "after", 5, 3, dev)
        line["qaoa"] = _public(measure_qaoa(24, 10, 24, "complex128", 5, 3, dev))
        # the largest configured size whose history does not fit: uncompute mode
        line["large"] = measure_mcclean(28, 50, 28, "complex128", "cnot", "before", 2, 2, dev, min_warmup=2)
        line["batched"] = measure_batched(14, 30, 4096, "complex64", 5, 3, 14, dev, e2e=True)
        # config 3's complex128 check: n = 14 complex128 jobs on 4-CTA clusters
        line["batched_c128"] = measure_batched(14, 30, 1024, "complex128", 3, 3, 14, dev, e2e=False)
        line["served"] = {"small": measure_served(24, 1000, 14, args.streams, dev),
                          "full": measure_served(26, 60, 26, args.streams, dev)}
        line["extras_clocks"] = extra_clk.stop()
        line["extras_wall_s"] = time.perf_counter() - t0
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.n, args.layers, axes, angles, args.cpu_layers)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""Time the reference's own numpy grad_run beside the C oracle, on this host.

Runs the unmodified ``qradient.circuit_logic`` McClean.grad_run of a
qradient checkout (through ``ref_shim.py``, as ``make_golden.py`` does)
and ``oracle/qg_oracle.c``'s grad_run on the same seeded circuits, so that
the CPU baseline the benchmark reports (the oracle on all host cores) can
be read against the reference itself (numpy and scipy, effectively one
core).  The reference cannot run where the GPU is, so this is run here.

Usage:  python tests/golden/time_reference.py --reference PATH [--max-n 18]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("QRADIENT_REFERENCE"))
    ap.add_argument("--max-n", type=int, default=18)
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference PATH (or QRADIENT_REFERENCE) is required")
    from make_golden import load_reference

    from oracle import oracle as O

    McClean, _ = load_reference(args.reference)
    print("n  L   reference numpy grad_run s   oracle grad_run s (%d threads)   ratio" % O.num_threads())
    for n, L in ((10, 10), (14, 30), (16, 50), (18, 50)):
        if n > args.max_n:
            continue
        rng = np.random.default_rng(n)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        zz = np.full((n, n), None)
        for i in range(n - 1):
            zz[i, i + 1] = 1.0
        c = McClean(n, {"zz": zz}, L, axes=axes, angles=angles)
        t0 = time.perf_counter()
        E_ref, g_ref = c.grad_run()
        t_ref = time.perf_counter() - t0
        t = O.Terms(np.full(n - 1, 3), np.arange(n - 1), np.arange(1, n), np.ones(n - 1))
        O.mcclean_grad(n, axes, angles, t)
        t0 = time.perf_counter()
        E, g = O.mcclean_grad(n, axes, angles, t)
        t_or = time.perf_counter() - t0
        assert abs(E - E_ref) < 1e-12 and np.max(np.abs(g - g_ref)) <= 1e-12 * max(np.max(np.abs(g_ref)), 1e-300)
        print("%2d %3d   %10.3f                   %10.4f                       %6.1f" % (n, L, t_ref, t_or, t_ref / t_or),
              flush=True)


if __name__ == "__main__":
    main()

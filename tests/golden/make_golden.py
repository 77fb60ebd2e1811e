"""Generate the golden vectors in ``tests/golden/`` from the reference itself.

Runs the reference's *unmodified* circuit logic
(``qradient/circuit_logic/mc_clean.py``, ``qaoa.py``, ``base.py``) from a
checkout given by ``--reference`` (default ``/root/reference``), with
``ref_shim.py`` standing in for the ``qradient.physical_components`` classes
the snapshot lacks.  Inputs are seeded (``numpy.random.default_rng``) and
stored beside the outputs, so the tests never need the reference.

Usage:  python tests/golden/make_golden.py [--reference PATH] [--big]

``--big`` adds the McClean ZZ-chain cases at n = 18, 20 (L = 50), which take
about two minutes of reference time.
"""
import argparse
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(path):
    sys.path.insert(0, path)
    spec = importlib.util.spec_from_file_location("qradient.physical_components", os.path.join(HERE, "ref_shim.py"))
    shim = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(shim)
    sys.modules["qradient.physical_components"] = shim
    from qradient.circuit_logic import McClean, Qaoa  # noqa: E402

    return McClean, Qaoa


def obs_to_arrays(n, obs):
    """Observable dict -> (kind, q0, q1, w) with kind 0..3 = X, Y, Z, ZZ."""
    kind, q0, q1, w = [], [], [], []
    for key, k in (("x", 0), ("y", 1), ("z", 2)):
        if key in obs:
            for q, v in enumerate(obs[key]):
                if v is not None:
                    kind.append(k), q0.append(q), q1.append(q), w.append(float(v))
    if "zz" in obs:
        for i in range(n):
            for j in range(i + 1, n):
                if obs["zz"][i, j] is not None:
                    kind.append(3), q0.append(i), q1.append(j), w.append(float(obs["zz"][i, j]))
    return (np.array(kind, np.int32), np.array(q0, np.int32), np.array(q1, np.int32), np.array(w, np.float64))


def zz_pairs(n, pairs, weight=1.0):
    zz = np.full((n, n), None)
    for i, j in pairs:
        zz[min(i, j), max(i, j)] = weight
    return zz


def regular3(n, seed):
    import networkx as nx

    g = nx.random_regular_graph(3, n, seed=seed)
    return sorted((min(a, b), max(a, b)) for a, b in g.edges())


def mcclean_cases(big):
    """(name, n, L, seed, observable, ladder, with_ini)"""
    cases = []
    for n, L in [(1, 3), (2, 1), (2, 4), (3, 0), (3, 2), (4, 3), (5, 5), (8, 6)]:
        obs = {"zz": zz_pairs(n, [(0, 1)])} if n >= 2 else {"z": np.array([1.0], dtype=object)}
        cases.append(("zz01_n%d_L%d" % (n, L), n, L, 100 + 7 * n + L, obs, "cnot", False))
    # the CPU configuration of the benchmark: n=10, L=10, Z0 Z1, seed 0
    cases.append(("config1_n10_L10", 10, 10, 0, {"zz": zz_pairs(10, [(0, 1)])}, "cnot", False))
    cases.append(("config1_cz_n10_L10", 10, 10, 0, {"zz": zz_pairs(10, [(0, 1)])}, "cz", False))
    cases.append(("cz_n6_L4", 6, 4, 11, {"zz": zz_pairs(6, [(0, 1), (2, 5)])}, "cz", False))
    # general Pauli-sum observables
    for n, L, seed in [(5, 4, 21), (7, 3, 22), (9, 2, 23)]:
        r = np.random.default_rng(seed + 1000)
        obs = {}
        for key in ("x", "y", "z"):
            arr = np.full(n, None)
            for q in r.choice(n, size=max(1, n // 3), replace=False):
                arr[q] = float(r.uniform(-1, 1))
            obs[key] = arr
        zz = np.full((n, n), None)
        for _ in range(n):
            i, j = sorted(r.choice(n, size=2, replace=False))
            zz[i, j] = float(r.uniform(-1, 1))
        obs["zz"] = zz
        cases.append(("pauli_n%d_L%d" % (n, L), n, L, seed, obs, "cnot", False))
    cases.append(("ini_n6_L3", 6, 3, 31, {"zz": zz_pairs(6, [(0, 1)])}, "cnot", True))
    sizes = [(12, 20), (14, 30), (16, 50)] + ([(18, 50), (20, 50)] if big else [])
    for n, L in sizes:
        obs = {"zz": zz_pairs(n, [(i, i + 1) for i in range(n - 1)])}
        cases.append(("chain_n%d_L%d" % (n, L), n, L, n, obs, "cnot", False))
    return cases


def qaoa_cases():
    """(name, n, p, seed, edges, z_weights, with_ini)"""
    cases = []
    for n, p, seed in [(4, 1, 1), (6, 1, 2), (6, 3, 3), (8, 4, 4), (10, 5, 5), (12, 3, 6), (14, 2, 7)]:
        cases.append(("reg3_n%d_p%d" % (n, p), n, p, seed, regular3(n, seed), None, False))
    # 10 random edges, as in the reference's benchmark script
    r = np.random.default_rng(12)
    alle = [(i, j) for i in range(12) for j in range(i + 1, 12)]
    e10 = [alle[k] for k in sorted(r.choice(len(alle), size=10, replace=False))]
    cases.append(("edges10_n12_p10", 12, 10, 12, e10, None, False))
    cases.append(("zfield_n6_p2", 6, 2, 13, regular3(6, 13), [0.5, None, -0.25, None, None, 1.0], False))
    cases.append(("ini_n6_p2", 6, 2, 14, regular3(6, 14), None, True))
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--big", action="store_true")
    args = ap.parse_args()
    McClean, Qaoa = load_reference(args.reference)

    out = {}
    manifest = {"mcclean": [], "qaoa": []}
    for name, n, L, seed, obs, ladder, with_ini in mcclean_cases(args.big):
        rng = np.random.default_rng(seed)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        ini = None
        if with_ini:
            v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
            ini = v / np.linalg.norm(v)
        t0 = time.time()
        c = McClean(n, obs, L, axes=axes, angles=angles)
        if ladder == "cz":
            c.state.gates.use_cz_ladder()
        e_run = c.run_expec_val(ini_state=None if ini is None else ini.copy())
        state = c.state.vec.copy() if n <= 8 else None
        e_grad, grad = c.grad_run(ini_state=None if ini is None else ini.copy())
        kind, q0, q1, w = obs_to_arrays(n, obs)
        key = "mcclean/" + name + "/"
        out.update({key + "axes": axes.astype(np.int8), key + "angles": angles, key + "kind": kind, key + "q0": q0,
                    key + "q1": q1, key + "w": w, key + "e_run": np.float64(e_run), key + "e_grad": np.float64(e_grad),
                    key + "grad": grad})
        if ini is not None:
            out[key + "ini"] = ini
        if state is not None:
            out[key + "state"] = state
        manifest["mcclean"].append({"name": name, "n": n, "L": L, "seed": seed, "ladder": ladder,
                                    "placement": "before", "ini": bool(with_ini)})
        print("mcclean %-22s %.2fs" % (name, time.time() - t0), flush=True)

    for name, n, p, seed, edges, zw, with_ini in qaoa_cases():
        rng = np.random.default_rng(seed)
        betas = rng.uniform(0, np.pi, p)
        gammas = rng.uniform(0, np.pi, p)
        obs = {"zz": zz_pairs(n, edges)}
        if zw is not None:
            obs["z"] = np.array(zw, dtype=object)
        ini = None
        if with_ini:
            v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
            ini = v / np.linalg.norm(v)
        t0 = time.time()
        c = Qaoa(n, obs, p)
        e_run = c.run_expec_val(betas, gammas, ini_state=None if ini is None else ini.copy())
        state = c.state.vec.copy() if n <= 8 else None
        e_grad, grad = c.grad_run(betas, gammas, ini_state=None if ini is None else ini.copy())
        kind, q0, q1, w = obs_to_arrays(n, obs)
        key = "qaoa/" + name + "/"
        out.update({key + "edges": np.array(edges, np.int32), key + "betas": betas, key + "gammas": gammas,
                    key + "kind": kind, key + "q0": q0, key + "q1": q1, key + "w": w,
                    key + "e_run": np.float64(e_run), key + "e_grad": np.float64(e_grad), key + "grad": grad})
        if n <= 12 and zw is None:
            ch = c.state.gates.classical_ham
            assert np.all(ch == np.round(ch))
            out[key + "cost_table"] = ch.astype(np.int32)
        if ini is not None:
            out[key + "ini"] = ini
        if state is not None:
            out[key + "state"] = state
        manifest["qaoa"].append({"name": name, "n": n, "p": p, "seed": seed, "ini": bool(with_ini)})
        print("qaoa    %-22s %.2fs" % (name, time.time() - t0), flush=True)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()

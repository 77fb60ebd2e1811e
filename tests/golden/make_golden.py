"""Generate the golden vectors in ``tests/golden/`` from the reference itself.

Runs the reference's *unmodified* circuit logic
(``qradient/circuit_logic/mc_clean.py``, ``qaoa.py``, ``base.py``) from a
checkout given by ``--reference`` (or the ``QRADIENT_REFERENCE`` environment
variable; one of the two is required), with
``ref_shim.py`` standing in for the ``qradient.physical_components`` classes
the snapshot lacks.  Inputs are seeded (``numpy.random.default_rng``) and
stored beside the outputs, so the tests never need the reference.

Usage:  python tests/golden/make_golden.py --reference PATH [--big]
        python tests/golden/make_golden.py --optimizer --reference PATH
        python tests/golden/make_golden.py --projectors --reference PATH
        python tests/golden/make_golden.py --ladder --reference PATH

``--big`` adds the McClean ZZ-chain cases at n = 18, 20 (L = 50), which take
about two minutes of reference time.

``--projectors`` writes ``projectors.npz``: the +1-projector probabilities
||Pi_+ psi||^2 of every observable term (the reference's ``Projector``,
``observable.py:126-177``, as ``sample_expec_val`` uses them,
``base.py:22-33``) on the golden final states of the Pauli-sum cases.

``--optimizer`` writes ``optimizer.npz`` instead: the reference's own
optimiser classes (``qradient/optimization.py``) fed seeded gradient and cost
sequences (the update rules alone), and ``McCleanOpt`` / ``QaoaOpt``
training runs with Adam, GradientDescent and RateDecayOnPlateau (the
histories of whole training loops).
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
    cases.append(("zz01_seed0_n10_L10", 10, 10, 0, {"zz": zz_pairs(10, [(0, 1)])}, "cnot", False))
    cases.append(("zz01_cz_seed0_n10_L10", 10, 10, 0, {"zz": zz_pairs(10, [(0, 1)])}, "cz", False))
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


def gd_decay(step_size, it):
    """Decay function of the GradientDescent golden cases (also in the tests)."""
    return step_size / (1.0 + 0.25 * it)


OPT_RULE_CASES = [
    # (name, optimizer dict, nparams, steps)
    ("adam_default", {"name": "Adam"}, 37, 30),
    ("adam_custom", {"name": "Adam", "step_size": 0.05, "beta1": 0.8, "beta2": 0.99, "eps": 1e-6}, 300, 25),
    ("gd_plain", {"name": "GradientDescent", "step_size": 0.1}, 37, 20),
    ("gd_decay", {"name": "GradientDescent", "step_size": 0.2, "decay_function": gd_decay}, 37, 20),
    ("plateau", {"name": "RateDecayOnPlateau", "step_size": 0.3, "plateau_length": 3, "decay_rate": 0.5}, 37, 40),
]

COMPONENT_CASES = [
    # (name, n, L, seed, draws): Pauli-sum observable with positive weights
    ("comp_n5_L3", 5, 3, 51, 6),
    ("comp_n7_L4", 7, 4, 52, 6),
]


def component_observable(n, seed):
    r = np.random.default_rng(seed + 2000)
    obs = {}
    for key in ("x", "y", "z"):
        arr = np.full(n, None)
        for q in r.choice(n, size=max(1, n // 2), replace=False):
            arr[q] = float(r.uniform(0.2, 1.0))
        obs[key] = arr
    obs["zz"] = zz_pairs(n, [(i, i + 1) for i in range(n - 1)], 0.7)
    return obs


OPT_RUN_CASES = [
    # (name, family, n, layers, optimizer dict, steps, seed)
    ("mcclean_adam_n6_L4", "mcclean", 6, 4, {"name": "Adam", "step_size": 0.05}, 15, 41),
    ("mcclean_gd_n5_L3", "mcclean", 5, 3, {"name": "GradientDescent", "step_size": 0.1,
                                           "decay_function": gd_decay}, 12, 42),
    ("mcclean_plateau_n6_L3", "mcclean", 6, 3, {"name": "RateDecayOnPlateau", "step_size": 0.9,
                                                "plateau_length": 2, "decay_rate": 0.5}, 20, 43),
    ("qaoa_adam_n8_p3", "qaoa", 8, 3, {"name": "Adam", "step_size": 0.05}, 15, 44),
    ("mcclean_adam_comp_n6_L3", "mcclean_comp", 6, 3, {"name": "Adam", "step_size": 0.05}, 12, 45),
]


def record(circuit, method):
    """Keep every gradient the optimiser's steps receive from `method`."""
    inner = getattr(circuit, method)
    circuit.recorded_grads = []

    def wrapped(*a, **k):
        e, g = inner(*a, **k)
        circuit.recorded_grads.append(np.array(g, dtype=np.float64))
        return e, g

    setattr(circuit, method, wrapped)


def optimizer_main(reference):
    McClean, Qaoa = load_reference(reference)
    from qradient import optimization as ropt

    out = {}
    for name, spec, npar, steps in OPT_RULE_CASES:
        rng = np.random.default_rng(len(name) * 101 + npar)
        p0 = rng.uniform(0, 2 * np.pi, npar)
        grads = rng.normal(size=(steps, npar)) * rng.uniform(1e-3, 2.0, (steps, 1))
        # costs that fall, then rise for a while, so the plateau rule decays the rate
        costs = np.cumsum(rng.normal(size=steps) + np.where(np.arange(steps) % 9 < 4, -0.5, 0.4))
        holder = ropt.ParametrizedCircuitOptimizer()
        holder.pick(spec, p0.copy())
        opt = holder.optimizer
        hist = np.zeros((steps + 1, npar))
        hist[0] = p0
        rates = np.zeros(steps)
        for k in range(steps):
            opt.step(grads[k], costs[k])
            hist[k + 1] = opt.parameters
            rates[k] = opt.step_size
        key = "rule/" + name + "/"
        out.update({key + "p0": p0, key + "grads": grads, key + "costs": costs, key + "hist": hist,
                    key + "rates": rates})
        print("rule   %-24s done" % name, flush=True)

    for name, n, L, seed, draws in COMPONENT_CASES:
        rng = np.random.default_rng(seed)
        obs = component_observable(n, seed)
        axes = rng.integers(0, 3, (L, n))
        angles = rng.uniform(0, 2 * np.pi, (L, n))
        c = McClean(n, obs, L, use_observable_components=True, axes=axes, angles=angles)
        np.random.seed(seed)
        es, gs = [], []
        for _ in range(draws):
            e, g = c.grad_run_with_component_sampling()
            es.append(e)
            gs.append(g.copy())
        kind, q0, q1, w = obs_to_arrays(n, obs)
        key = "comp/" + name + "/"
        out.update({key + "axes": axes.astype(np.int8), key + "angles": angles, key + "kind": kind, key + "q0": q0,
                    key + "q1": q1, key + "w": w, key + "e": np.array(es), key + "grads": np.array(gs)})
        print("comp   %-24s done" % name, flush=True)

    for name, fam, n, layers, spec, steps, seed in OPT_RUN_CASES:
        rng = np.random.default_rng(seed)
        key = "run/" + name + "/"
        t0 = time.time()
        if fam in ("mcclean", "mcclean_comp"):
            comp = fam == "mcclean_comp"
            if comp:
                obs = component_observable(n, seed)
            else:
                obs = {"zz": zz_pairs(n, [(i, i + 1) for i in range(n - 1)]),
                       "x": np.array([0.5] + [None] * (n - 1), dtype=object)}
            axes = rng.integers(0, 3, (layers, n))
            angles = rng.uniform(0, 2 * np.pi, (layers, n))
            c = McClean(n, obs, layers, use_observable_components=comp, axes=axes, angles=angles.copy())
            record(c, "grad_run_with_component_sampling" if comp else "grad_run")
            o = ropt.McCleanOpt(c, spec, max_iter=steps + 1)
            np.random.seed(seed)
            for _ in range(steps):
                o.step(component_sampling=comp)
            out.update({key + "axes": axes.astype(np.int8), key + "angles": angles})
        else:
            edges = regular3(n, seed)
            obs = {"zz": zz_pairs(n, edges)}
            betas = rng.uniform(0, np.pi, layers)
            gammas = rng.uniform(0, np.pi, layers)
            c = Qaoa(n, obs, layers)
            record(c, "grad_run")
            o = ropt.QaoaOpt(c, spec, betas, gammas, max_iter=steps + 1)
            for _ in range(steps):
                o.step()
            out.update({key + "edges": np.array(edges, np.int32), key + "betas": betas, key + "gammas": gammas})
        kind, q0, q1, w = obs_to_arrays(n, obs)
        out.update({key + "kind": kind, key + "q0": q0, key + "q1": q1, key + "w": w,
                    key + "param_history": o.param_history, key + "cost_history": o.cost_history,
                    key + "grads": np.array(c.recorded_grads)})
        print("run    %-24s %.2fs" % (name, time.time() - t0), flush=True)

    np.savez_compressed(os.path.join(HERE, "optimizer.npz"), **out)
    print("wrote", len(out), "arrays to optimizer.npz")


def projectors_main(reference):
    """Projector probabilities from the reference's Projector class.  The
    snapshot's Observable.load_projectors calls a method that does not exist
    (observable.py:85 calls check_observable; the method is the name-mangled
    __check_observable of :106), so the projectors are built here in the
    order load_projectors would build them (observable.py:88-103)."""
    spec = importlib.util.spec_from_file_location(
        "ref_observable", os.path.join(reference, "qradient", "physical_components", "observable.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    Projector = mod.Projector
    gold = np.load(os.path.join(HERE, "golden.npz"))
    out = {}
    names = sorted({k.split("/")[1] for k in gold.files if k.startswith("mcclean/") and k.endswith("/state")})
    for name in names:
        key = "mcclean/" + name + "/"
        kind, q0, q1, vec = gold[key + "kind"], gold[key + "q0"], gold[key + "q1"], gold[key + "state"]
        n = int(np.log2(vec.size))
        Projector.set_qnum(n)
        probs = []
        for k, a, b in zip(kind, q0, q1):
            key_id = "xyz"[k] if k < 3 else "zz"
            proj = Projector(key_id, int(a)) if k < 3 else Projector("zz", int(a), int(b))
            probs.append((np.abs(proj.dot(vec)) ** 2).sum())
        out[name + "/p_plus"] = np.array(probs)
        print("projectors %-22s %d terms" % (name, len(probs)), flush=True)
    np.savez_compressed(os.path.join(HERE, "projectors.npz"), **out)
    print("wrote", len(out), "arrays to projectors.npz")


def ladder_main(reference):
    """The reference's CNOT ladders, periodic and open, as they act on seeded
    random states: State.load_cnot_ladder(periodic) (state.py:209-241) built
    by the reference's own State class and applied through its stored
    matrices (the method cnot_ladder shadows them, state.py:243-251, so they
    are read as State._State__cnot_ladder).  McClean builds only the open
    ladder; the periodic one is the reference's other ladder option."""
    spec = importlib.util.spec_from_file_location(
        "ref_state", os.path.join(reference, "qradient", "physical_components", "state.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    rng = np.random.default_rng(2024)
    for n in (2, 4, 6, 8, 10):
        st = mod.State(n)
        for periodic in (True, False):
            st.load_cnot_ladder(periodic=periodic)
            mats = st._State__cnot_ladder
            v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
            tag = "n%d/%s/" % (n, "periodic" if periodic else "open")
            out[tag + "in"] = v
            out[tag + "stack0"] = mats[0].dot(v)
            out[tag + "stack1"] = mats[1].dot(v)
        print("ladder n=%d" % n, flush=True)
    try:
        mod.State(5).load_cnot_ladder(periodic=True)
        out["odd_n_raises"] = np.array(False)
    except ValueError:
        out["odd_n_raises"] = np.array(True)
    np.savez_compressed(os.path.join(HERE, "ladder.npz"), **out)
    print("wrote", len(out), "arrays to ladder.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("QRADIENT_REFERENCE"),
                    help="path of a qradient checkout (or set QRADIENT_REFERENCE)")
    ap.add_argument("--big", action="store_true")
    ap.add_argument("--optimizer", action="store_true")
    ap.add_argument("--projectors", action="store_true")
    ap.add_argument("--ladder", action="store_true")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference PATH (or QRADIENT_REFERENCE) is required")
    if args.projectors:
        return projectors_main(args.reference)
    if args.ladder:
        return ladder_main(args.reference)
    if args.optimizer:
        return optimizer_main(args.reference)
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

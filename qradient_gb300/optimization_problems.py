"""Problem generators feeding the QAOA circuit
(counterpart of ``qradient/optimization_problems.py``).

``MaxCut(vertex_num, edge_set=... | edge_num=... | edge_probability=...)``
and ``to_observable()`` follow optimization_problems.py:3-37 (zz[i, j] = 1
for every edge, i < j).  ``random_regular_edges`` draws a seeded random
d-regular graph with the pairing (configuration) model and rejection of
self-loops and multi-edges, so that benchmark graphs can be generated on
machines without networkx.
"""
import numpy as np


class MaxCut:
    def __init__(self, vertex_num, **kwargs):
        self.vertex_num = vertex_num
        if "edge_set" in kwargs:
            self.edge_set = np.asarray(kwargs["edge_set"])
        elif "edge_num" in kwargs:
            self._random(edge_num=kwargs["edge_num"])
        elif "edge_probability" in kwargs:
            self._random(edge_probability=kwargs["edge_probability"])
        else:
            raise ValueError("Specify one of the three edge_set, edge_num, or edge_probability")

    def _random(self, **kwargs):
        all_edges = np.array([[i, j] for i in range(self.vertex_num) for j in range(i + 1, self.vertex_num)])
        if "edge_num" in kwargs:
            idx = np.random.choice(range(len(all_edges)), size=kwargs["edge_num"], replace=False)
            self.edge_set = all_edges[idx]
        else:
            keep = [e for e in all_edges if np.random.rand() < kwargs["edge_probability"]]
            self.edge_set = np.array(keep)

    def to_observable(self):
        zz = np.full([self.vertex_num, self.vertex_num], None)
        for e in self.edge_set:
            i, j = int(min(e)), int(max(e))
            zz[i, j] = 1.0
        return {"zz": zz}


def random_regular_edges(degree, n, seed, max_tries=10000):
    """Edges (i < j, sorted) of a random simple degree-regular graph on n nodes."""
    if (degree * n) % 2 or degree >= n:
        raise ValueError("no %d-regular graph on %d nodes" % (degree, n))
    rng = np.random.default_rng(seed)
    for _ in range(max_tries):
        stubs = np.repeat(np.arange(n), degree)
        rng.shuffle(stubs)
        pairs = stubs.reshape(-1, 2)
        a, b = np.minimum(pairs[:, 0], pairs[:, 1]), np.maximum(pairs[:, 0], pairs[:, 1])
        if np.any(a == b):
            continue
        key = a * n + b
        if len(np.unique(key)) != len(key):
            continue
        order = np.argsort(key)
        return np.stack([a[order], b[order]], axis=1)
    raise RuntimeError("could not draw a simple regular graph")

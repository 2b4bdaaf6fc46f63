"""Generates tests/golden/triangles.json — run from the repo root:

    python tests/golden/make_golden.py

Each case is a small undirected graph (edge list, possibly with duplicates
and self loops, as generators emit them) with:
  * ``triangles``: networkx 3.6.1 ``sum(nx.triangles(G).values()) // 3``
  * ``analytic``: the closed-form count where one exists (K_n, K_{a,b}, wheels,
    grids, Petersen, disjoint unions), else null
  * ``per_vertex``: networkx per-vertex triangle counts
  * ``oriented_per_edge``: |N+(u) n N+(v)| for every oriented edge u->v of the
    degree-ordered DAG (keep u->v iff deg(v) > deg(u) or equal degree and
    v > u), rows by u ascending and neighbours ascending, computed here with
    networkx DiGraph successor sets.
The random cases use numpy's seeded generator, independent of the engine's
own generators.
"""
from __future__ import annotations

import json
from math import comb
from pathlib import Path

import networkx as nx
import numpy as np


def case(name, n, edges, analytic=None):
    G = nx.Graph()
    G.add_nodes_from(range(n))
    G.add_edges_from((int(u), int(v)) for u, v in edges if u != v)
    tri = nx.triangles(G)
    total = sum(tri.values()) // 3
    if analytic is not None:
        assert total == analytic, (name, total, analytic)
    deg = dict(G.degree())
    D = nx.DiGraph()
    D.add_nodes_from(range(n))
    for u, v in G.edges():
        a, b = (u, v) if (deg[v] > deg[u] or (deg[v] == deg[u] and v > u)) else (v, u)
        D.add_edge(a, b)
    per_edge = []
    for u in range(n):
        su = set(D.successors(u))
        for v in sorted(su):
            per_edge.append(len(su & set(D.successors(v))))
    assert sum(per_edge) == total
    return {"name": name, "n": n, "edges": [[int(u), int(v)] for u, v in edges], "triangles": total,
            "analytic": analytic, "per_vertex": [tri[v] for v in range(n)], "oriented_per_edge": per_edge}


def main():
    cases = []
    for k in range(1, 13):
        cases.append(case(f"K{k}", k, [(i, j) for i in range(k) for j in range(i + 1, k)], comb(k, 3)))
    for a, b in [(1, 1), (2, 3), (4, 4), (5, 7)]:
        cases.append(case(f"K{a},{b}", a + b, [(i, a + j) for i in range(a) for j in range(b)], 0))
    for k in [3, 4, 5, 8, 17]:
        edges = [(0, 1 + i) for i in range(k)] + [(1 + i, 1 + (i + 1) % k) for i in range(k)]
        cases.append(case(f"wheel{k}", k + 1, edges, k if k >= 4 else 4))
    for r, c in [(2, 2), (3, 5), (10, 10)]:
        edges = [(i * c + j, i * c + j + 1) for i in range(r) for j in range(c - 1)] + \
                [(i * c + j, (i + 1) * c + j) for i in range(r - 1) for j in range(c)]
        cases.append(case(f"grid{r}x{c}", r * c, edges, 0))
    P = nx.petersen_graph()
    cases.append(case("petersen", 10, list(P.edges()), 0))
    # disjoint union K5 + K4 + wheel6: additive
    edges = [(i, j) for i in range(5) for j in range(i + 1, 5)]
    edges += [(5 + i, 5 + j) for i in range(4) for j in range(i + 1, 4)]
    edges += [(9, 10 + i) for i in range(6)] + [(10 + i, 10 + (i + 1) % 6) for i in range(6)]
    cases.append(case("union_K5_K4_wheel6", 16, edges, 10 + 4 + 6))
    cases.append(case("empty5", 5, [], 0))
    cases.append(case("single_vertex", 1, [], 0))
    cases.append(case("self_loops_and_dups", 4, [(0, 0), (0, 1), (1, 0), (1, 2), (2, 0), (0, 1), (3, 3)], 1))
    rng = np.random.default_rng(20261203)
    for i, (n, m) in enumerate([(30, 120), (64, 400), (200, 1500), (500, 6000), (1000, 12000)]):
        e = rng.integers(0, n, size=(m, 2))
        cases.append(case(f"er_{n}_{m}_{i}", n, e.tolist()))
    # skewed: preferential attachment with a hub
    for n, k in [(300, 3), (1500, 5)]:
        G = nx.barabasi_albert_graph(n, k, seed=7)
        cases.append(case(f"ba_{n}_{k}", n, list(G.edges())))
    # small R-MAT-like sample drawn with numpy (a=0.57, b=0.19, c=0.19)
    for scale, ef in [(8, 8), (10, 8)]:
        n = 1 << scale
        m = ef * n
        u = np.zeros(m, np.int64)
        v = np.zeros(m, np.int64)
        for _ in range(scale):
            r = rng.random(m)
            bu = (r >= 0.76).astype(np.int64)
            bv = (((r >= 0.57) & (r < 0.76)) | (r >= 0.95)).astype(np.int64)
            u = u * 2 + bu
            v = v * 2 + bv
        cases.append(case(f"rmat_s{scale}_ef{ef}", n, np.stack([u, v], 1).tolist()))
    out = Path(__file__).resolve().parent / "triangles.json"
    out.write_text(json.dumps({"generator": "tests/golden/make_golden.py", "networkx": nx.__version__,
                               "cases": cases}, separators=(",", ":")))
    print(f"wrote {out} ({out.stat().st_size} bytes, {len(cases)} cases)")


if __name__ == "__main__":
    main()

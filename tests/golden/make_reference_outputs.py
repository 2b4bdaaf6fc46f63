"""Generates tests/golden/reference_outputs.json from the reference's own
code — run from the repo root where the reference tree is present:

    bash oracle/build_ref.sh && python tests/golden/make_reference_outputs.py

oracle/_ref/libtc_ref.so is the reference's successful_push_pull/graph.cc,
compiled unchanged (oracle/build_ref.sh).  For every graph below it records
what the reference computes:
  * Graph::Graph(prefix, use_dag=true) -> Graph::orientation
    (graph.cc:252-298): the oriented rowptr/colidx;
  * Graph::intersect_num(u, v, label) (graph.cc:376-391) over every oriented
    edge, summed as bs_warp_vertex.cuh:13-21 does: per-edge counts and total;
  * for the labelled cases, the same with labels read from prefix.vlabel.bin;
  * for the unsorted case, the order of main.cc:19-31 with adj_sorted=0:
    the constructor orients the rows in file order, then
    Graph::sort_neighbors (graph.cc:156-164) sorts every DAG row.
Arrays are stored as sha256 digests of their little-endian bytes (int64
rowptr, int32 colidx, uint32 per-edge counts), totals as integers.

Graphs: the golden cases of triangles.json that the reference accepts
(Graph::Graph asserts 0 < max_degree < n, graph.cc:47), and seeded graphs
drawn here with a splitmix64 stream in numpy (identical on every machine):
Erdos-Renyi n=16384 average degree 16 (the small plain-method workload),
R-MAT scale 14 and 16 (a, b, c) = (0.57, 0.19, 0.19), a star-heavy graph
with hubs, and labelled variants.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser of x (uint64 array, wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, count: int) -> np.ndarray:
    """count doubles in [0, 1) from counter (seed, stream, i)."""
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed) * np.uint64(0x100000001B3) + np.uint64(stream))
        x = splitmix64(np.arange(count, dtype=np.uint64) + key)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def symmetric_csr(n: int, u: np.ndarray, v: np.ndarray):
    """Symmetrise, drop self loops, dedup, sort rows (numpy only)."""
    u = np.asarray(u, np.int64)
    v = np.asarray(v, np.int64)
    keep = u != v
    a = np.concatenate([u[keep], v[keep]])
    b = np.concatenate([v[keep], u[keep]])
    key = np.unique(a * n + b)
    src = key // n
    col = (key % n).astype(np.int32)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, src + 1, 1)
    return np.cumsum(rowptr).astype(np.int64), col


def er(n: int, avg_degree: float, seed: int):
    m = int(n * avg_degree / 2)
    u = np.minimum((uniform(seed, 0, m) * n).astype(np.int64), n - 1)
    v = np.minimum((uniform(seed, 1, m) * n).astype(np.int64), n - 1)
    return symmetric_csr(n, u, v)


def rmat(scale: int, edge_factor: int, seed: int, a=0.57, b=0.19, c=0.19):
    n = 1 << scale
    m = edge_factor * n
    u = np.zeros(m, np.int64)
    v = np.zeros(m, np.int64)
    for lvl in range(scale):
        r = uniform(seed, 2 + lvl, m)
        bu = (r >= a + b).astype(np.int64)
        bv = (((r >= a) & (r < a + b)) | (r >= a + b + c)).astype(np.int64)
        u = u * 2 + bu
        v = v * 2 + bv
    return symmetric_csr(n, u, v)


def hubs(n: int, seed: int):
    """A few hubs joined to most vertices plus a sparse random background:
    oriented rows far longer than 512 entries at the hubs' neighbours."""
    k = 8
    hu = np.repeat(np.arange(k), n // 2)
    hv = np.minimum((uniform(seed, 40, k * (n // 2)) * n).astype(np.int64), n - 1)
    m = 4 * n
    u = np.minimum((uniform(seed, 41, m) * n).astype(np.int64), n - 1)
    v = np.minimum((uniform(seed, 42, m) * n).astype(np.int64), n - 1)
    clique = np.arange(k, k + 700)
    cu, cv = np.meshgrid(clique, clique)
    sel = cu < cv
    return symmetric_csr(n, np.concatenate([hu, u, cu[sel]]), np.concatenate([hv, v, cv[sel]]))


def labels_for(n: int, classes: int, seed: int) -> np.ndarray:
    return np.minimum((uniform(seed, 99, n) * classes).astype(np.int64), classes - 1).astype(np.uint8)


def shuffled_rows(rowptr, colidx, seed: int):
    """The same graph with every row's entries in a seeded random order."""
    col = colidx.copy()
    r = uniform(seed, 77, len(col))
    for u in range(len(rowptr) - 1):
        s, e = rowptr[u], rowptr[u + 1]
        col[s:e] = col[s:e][np.argsort(r[s:e], kind="stable")]
    return col


def seeded_graphs():
    """name -> (rowptr, colidx, labels or None, label classes, sort_neighbors)."""
    g = {}
    g["er_n16384_d16_seed0"] = (*er(16384, 16, 0), None, 0, False)
    g["er_n4096_d32_seed3"] = (*er(4096, 32, 3), None, 0, False)
    g["rmat_s14_ef16_seed1"] = (*rmat(14, 16, 1), None, 0, False)
    g["rmat_s16_ef16_seed2"] = (*rmat(16, 16, 2), None, 0, False)
    g["hubs_n20000_seed4"] = (*hubs(20000, 4), None, 0, False)
    rp, col = rmat(12, 16, 5)
    g["rmat_s12_ef16_seed5_labels4"] = (rp, col, labels_for(len(rp) - 1, 4, 5), 4, False)
    rp, col = er(3000, 24, 6)
    g["er_n3000_d24_seed6_labels3"] = (rp, col, labels_for(len(rp) - 1, 3, 6), 3, False)
    rp, col = rmat(11, 16, 7)
    g["rmat_s11_ef16_seed7_unsorted"] = (rp, shuffled_rows(rp, col, 7), None, 0, True)
    return g


def digest(a: np.ndarray, dtype) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype).tobytes()).hexdigest()


def record(name, rowptr, colidx, labels, classes, sort_neighbors):
    from oracle import ref
    out = {"name": name, "n": int(len(rowptr) - 1), "nnz": int(len(colidx)), "sort_neighbors": sort_neighbors,
           "input_rowptr_sha256": digest(rowptr, np.int64), "input_colidx_sha256": digest(colidx, np.int32)}
    with ref.RefGraph(rowptr, colidx, labels=labels, sort_neighbors=sort_neighbors) as g:
        orow, ocol = g.arrays()
        out["m"] = g.m
        out["max_out_degree"] = g.max_degree
        out["dag_rowptr_sha256"] = digest(orow, np.int64)
        out["dag_colidx_sha256"] = digest(ocol, np.int32)
        if labels is None:
            t, pe = g.count(label=0, per_edge=True)
            out["total"] = t
            out["per_edge_sha256"] = digest(pe, np.uint32)
        else:
            out["labels_sha256"] = digest(labels, np.uint8)
            out["labelled"] = []
            for lab in range(classes):
                t, pe = g.count(label=lab, per_edge=True)
                out["labelled"].append({"label": lab, "total": t, "per_edge_sha256": digest(pe, np.uint32)})
    return out


def golden_csr(case):
    e = np.array(case["edges"], np.int64).reshape(-1, 2)
    return symmetric_csr(case["n"], e[:, 0], e[:, 1])


def main():
    from oracle import ref
    if not ref.available():
        raise SystemExit("oracle/_ref is not built: the reference tree is needed to make these fixtures")
    cases = json.loads((Path(__file__).resolve().parent / "triangles.json").read_text())["cases"]
    out = {"generator": "tests/golden/make_reference_outputs.py",
           "reference": "successful_push_pull/graph.cc (Graph::Graph, orientation, sort_neighbors, "
                        "intersect_num) compiled unchanged by oracle/build_ref.sh",
           "golden": [], "seeded": []}
    for c in cases:
        rp, col = golden_csr(c)
        if not ref.accepts(rp):
            out["golden"].append({"name": c["name"], "rejected_by_reference": "Graph::Graph asserts "
                                  "0 < max_degree < n (graph.cc:47)"})
            continue
        out["golden"].append(record(c["name"], rp, col, None, 0, False))
    for name, (rp, col, lab, classes, srt) in seeded_graphs().items():
        out["seeded"].append(record(name, rp, col, lab, classes, srt))
        print(name, out["seeded"][-1].get("total"), out["seeded"][-1]["m"], file=sys.stderr)
    path = Path(__file__).resolve().parent / "reference_outputs.json"
    path.write_text(json.dumps(out, indent=1))
    print(f"wrote {path} ({path.stat().st_size} bytes)")


if __name__ == "__main__":
    main()

"""CPU oracle loader — TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
leg, always as the checker (or as the timed CPU reference); the engine never
imports it.  Wraps oracle/_build/libtc_oracle.so (tc_oracle.c, a plain C +
OpenMP restatement of the reference CPU path) and adds pure-Python helpers
for tiny graphs.

Parity status: pinned to the reference's own graph.cc.  oracle/_ref is
that file compiled unchanged (oracle/build_ref.sh, oracle/ref.py); the
restatement gives the same oriented arrays, per-edge, total and labelled
counts as it (tests/test_ref_pin.py), and the fixtures it produced are
committed in tests/golden/reference_outputs.json.  The reference's device
intersection (GraphMiner's intersect_num) is not vendored; its CPU merge
(graph.cc:376-391) is what both compute.  Also pinned to networkx, analytic
answers and brute force (tests/golden/triangles.json).
"""
from __future__ import annotations

import ctypes as C
import itertools
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "libtc_oracle.so"
GEN_HEADER = HERE.parent / "hetegeneous_parallel_programming_gb300" / "csrc" / "tc_gen_common.h"
_lib = None


def build() -> Path:
    subprocess.run(["bash", str(HERE / "build_oracle.sh")], check=True)
    return SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        srcs = [HERE / "tc_oracle.c", HERE / "build_oracle.sh", GEN_HEADER]
        if not SO.exists() or any(SO.stat().st_mtime < f.stat().st_mtime for f in srcs if f.exists()):
            build()
        h = C.CDLL(str(SO))
        P, I64 = C.c_void_p, C.c_int64
        h.oracle_orient.restype = I64
        h.oracle_orient.argtypes = [I64, P, P, P, P]
        h.oracle_count.restype = C.c_uint64
        h.oracle_count.argtypes = [I64, P, P, P]
        h.oracle_count_labelled.restype = C.c_uint64
        h.oracle_count_labelled.argtypes = [I64, P, P, P, C.c_int, P]
        h.oracle_count_vertices.restype = C.c_uint64
        h.oracle_count_vertices.argtypes = [I64, P, P, P]
        h.oracle_count_rows.restype = C.c_uint64
        h.oracle_count_rows.argtypes = [I64, P, P, I64, I64, I64, P]
        h.oracle_orient_rows_cost.restype = I64
        h.oracle_orient_rows_cost.argtypes = [I64, P, P, I64]
        h.oracle_sort_neighbors.restype = None
        h.oracle_sort_neighbors.argtypes = [I64, P, P]
        h.oracle_csr_from_edges.restype = I64
        h.oracle_csr_from_edges.argtypes = [I64, I64, P, P, P, P]
        h.oracle_batch_count.restype = None
        h.oracle_batch_count.argtypes = [I64, P, P, P, P]
        h.oracle_gen_num_samples.restype = I64
        h.oracle_gen_num_samples.argtypes = [C.c_int32, I64, C.c_int32, C.c_double, C.c_double]
        h.oracle_gen_edges.restype = I64
        h.oracle_gen_edges.argtypes = [C.c_int32, I64, C.c_int32] + [C.c_double] * 6 + [C.c_uint64, P, P, I64]
        h.oracle_max_threads.restype = C.c_int
        h.oracle_set_threads.argtypes = [C.c_int]
        _lib = h
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def orient(rowptr, colidx):
    """graph.cc:252-298 -> (dag_rowptr, dag_colidx)."""
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    colidx = np.ascontiguousarray(colidx, np.int32)
    n = len(rowptr) - 1
    orow = np.empty(n + 1, np.int64)
    ocol = np.empty(max(len(colidx), 1), np.int32)
    m = lib().oracle_orient(n, _p(rowptr), _p(colidx), _p(orow), _p(ocol))
    return orow, ocol[:m].copy()


def count(dag_rowptr, dag_colidx, per_edge: bool = False):
    """bs_warp_vertex.cuh:13-21 with the merge of graph.cc:376-391 -> (total, per-edge or None)."""
    dag_rowptr = np.ascontiguousarray(dag_rowptr, np.int64)
    dag_colidx = np.ascontiguousarray(dag_colidx, np.int32)
    n = len(dag_rowptr) - 1
    out = np.zeros(max(len(dag_colidx), 1), np.uint32) if per_edge else None
    t = lib().oracle_count(n, _p(dag_rowptr), _p(dag_colidx), _p(out) if per_edge else None)
    return int(t), (out[:len(dag_colidx)] if per_edge else None)


def count_sample(dag_rowptr, dag_colidx, row_step: int):
    """Counting restricted to rows 0, row_step, 2*row_step, ... (bounded CPU baseline)."""
    n = len(dag_rowptr) - 1
    return int(lib().oracle_count_rows(n, _p(dag_rowptr), _p(dag_colidx), 0, n, int(row_step), None))


def orient_sample_cost(rowptr, colidx, row_step: int) -> int:
    n = len(rowptr) - 1
    return int(lib().oracle_orient_rows_cost(n, _p(rowptr), _p(colidx), int(row_step)))


def labelled(rowptr, colidx, labels, label: int, per_edge: bool = False):
    """Orient, then graph.cc:376-391 with the label test on every oriented edge -> (total, per-edge or None)."""
    orow, ocol = orient(rowptr, colidx)
    n = len(orow) - 1
    labels = np.ascontiguousarray(labels, np.uint8)
    out = np.zeros(max(len(ocol), 1), np.uint32) if per_edge else None
    total = lib().oracle_count_labelled(n, _p(orow), _p(ocol), _p(labels), int(label), _p(out) if per_edge else None)
    return int(total), (out[:len(ocol)] if per_edge else None)


def vertex_triangles(rowptr, colidx):
    """Triangles through every vertex of a symmetric CSR (orient, then the
    merge of graph.cc:376-391 enumerating common neighbours) -> (total, uint64[n])."""
    orow, ocol = orient(rowptr, colidx)
    n = len(orow) - 1
    t = np.zeros(max(n, 1), np.uint64)
    total = lib().oracle_count_vertices(n, _p(orow), _p(ocol), _p(t))
    return int(total), t[:n]


def partition_totals(dag_rowptr, dag_colidx, part, num_parts: int, rule: str = "source"):
    """Per-PE partial counts of the reference's partitioned solver
    (successful_push_pull/bs_warp_vertex_nvshmem.cuh) on an oriented graph:
    every PE walks its own vertices u (:25-29); an edge u->v inside the
    partition is counted there (:36-38); a cross-partition edge is pulled
    and counted by part[u] when d+(u) >= d+(v), else pushed to and counted
    by part[v] (:127-136, receiver :224-232).  rule "source" credits every
    edge to part[u].  -> (total, uint64[num_parts])."""
    dag_rowptr = np.ascontiguousarray(dag_rowptr, np.int64)
    dag_colidx = np.ascontiguousarray(dag_colidx, np.int32)
    part = np.asarray(part, np.int64)
    total, pe = count(dag_rowptr, dag_colidx, per_edge=True)
    dplus = np.diff(dag_rowptr)
    src = np.repeat(np.arange(len(dplus)), dplus)
    dst = dag_colidx.astype(np.int64)
    credit = part[src].copy()
    if rule == "push_pull":
        push = (part[dst] != part[src]) & (dplus[src] < dplus[dst])
        credit[push] = part[dst][push]
    elif rule != "source":
        raise ValueError(rule)
    out = np.zeros(num_parts, np.uint64)
    np.add.at(out, credit, pe.astype(np.uint64))
    return total, out


def py_partition_totals(dag_rowptr, dag_colidx, part, num_parts: int, rule: str = "source"):
    """partition_totals stated as the PE loops themselves, in pure Python
    (small graphs only): PE p walks u in its vertex list, v in N+(u)."""
    n = len(dag_rowptr) - 1
    rows = [set(int(x) for x in dag_colidx[dag_rowptr[u]:dag_rowptr[u + 1]]) for u in range(n)]
    out = [0] * num_parts
    for p in range(num_parts):
        for u in (x for x in range(n) if part[x] == p):
            for v in dag_colidx[dag_rowptr[u]:dag_rowptr[u + 1]]:
                c = len(rows[u] & rows[int(v)])
                if rule == "push_pull" and part[v] != p and len(rows[u]) < len(rows[int(v)]):
                    out[int(part[v])] += c  # pushed: the receiver on part[v] counts it
                else:
                    out[p] += c
    return sum(out), out


def triangles(rowptr, colidx, per_edge: bool = False):
    """Full CPU path: orient then count."""
    orow, ocol = orient(rowptr, colidx)
    t, pe = count(orow, ocol, per_edge)
    return (t, pe, orow, ocol) if per_edge else t


def csr_from_edges(n: int, src, dst):
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    rowptr = np.empty(n + 1, np.int64)
    colidx = np.empty(max(2 * len(src), 1), np.int32)
    nnz = lib().oracle_csr_from_edges(n, len(src), _p(src), _p(dst), _p(rowptr), _p(colidx))
    if nnz < 0:
        raise ValueError("bad edge list")
    return rowptr, colidx[:nnz].copy()


GEN_KINDS = {"er": 0, "rmat": 1, "chung_lu": 3}


def gen_edges(kind: str, n: int = 0, scale: int = 0, avg_degree: float = 0.0, edge_factor: float = 16.0,
              a: float = 0.57, b: float = 0.19, c: float = 0.19, gamma: float = 2.1, seed: int = 0):
    """The engine's seeded samples (ER, R-MAT, Chung-Lu) drawn without the
    engine: (n, src, dst).  R-MAT has n = 2^scale."""
    k = GEN_KINDS[kind]
    if k == 1:
        n = 1 << scale
    M = int(lib().oracle_gen_num_samples(k, int(n), int(scale), float(avg_degree), float(edge_factor)))
    src = np.empty(max(M, 1), np.int32)
    dst = np.empty(max(M, 1), np.int32)
    got = lib().oracle_gen_edges(k, int(n), int(scale), float(avg_degree), float(edge_factor), float(a), float(b),
                                 float(c), float(gamma), int(seed), _p(src), _p(dst), M)
    if got != M:
        raise ValueError("bad generator parameters")
    return int(n), src[:M], dst[:M]


def batch_count(vtx_off, rowptr, colidx):
    vtx_off = np.ascontiguousarray(vtx_off, np.int64)
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    colidx = np.ascontiguousarray(colidx, np.int32)
    out = np.zeros(len(vtx_off) - 1, np.uint64)
    lib().oracle_batch_count(len(vtx_off) - 1, _p(vtx_off), _p(rowptr), _p(colidx), _p(out))
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def set_threads(t: int) -> None:
    lib().oracle_set_threads(int(t))


# ---- pure Python, tiny graphs -----------------------------------------------------------

def brute_force_triangles(n: int, edges) -> int:
    """Enumerate vertex triples (graphs of a few dozen vertices at most)."""
    adj = [set() for _ in range(n)]
    for u, v in edges:
        if u != v:
            adj[u].add(v)
            adj[v].add(u)
    return sum(1 for a, b, c in itertools.combinations(range(n), 3) if b in adj[a] and c in adj[a] and c in adj[b])


def py_orient_count(rowptr, colidx):
    """Independent pure-Python statement of orientation + per-edge counts."""
    n = len(rowptr) - 1
    deg = [int(rowptr[v + 1] - rowptr[v]) for v in range(n)]
    out_rows = []
    for u in range(n):
        out_rows.append([int(v) for v in colidx[rowptr[u]:rowptr[u + 1]]
                         if deg[v] > deg[u] or (deg[v] == deg[u] and v > u)])
    sets = [set(r) for r in out_rows]
    per = [len(sets[u] & sets[v]) for u in range(n) for v in out_rows[u]]
    return sum(per), per, out_rows

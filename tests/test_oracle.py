"""The CPU oracle pinned against golden vectors (networkx, analytic answers,
brute force) — no GPU needed."""
import itertools

import numpy as np
import pytest

from oracle import oracle


def csr_of(case):
    e = np.array(case["edges"], np.int64).reshape(-1, 2)
    return oracle.csr_from_edges(case["n"], e[:, 0], e[:, 1])


def test_golden_totals_and_per_edge(golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        total, per_edge, orow, ocol = oracle.triangles(rowptr, colidx, per_edge=True)
        assert total == case["triangles"], case["name"]
        if case["analytic"] is not None:
            assert total == case["analytic"], case["name"]
        assert per_edge.tolist() == case["oriented_per_edge"], case["name"]
        assert int(per_edge.sum()) == total


def test_orientation_rule_matches_python_statement(golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        orow, ocol = oracle.orient(rowptr, colidx)
        t, per, rows = oracle.py_orient_count(rowptr, colidx)
        assert [ocol[orow[u]:orow[u + 1]].tolist() for u in range(len(rowptr) - 1)] == rows
        assert t == case["triangles"]
        # every undirected edge kept exactly once
        assert len(ocol) * 2 == len(colidx)


def test_exhaustive_six_vertex_graphs():
    pairs = list(itertools.combinations(range(6), 2))
    for mask in range(1 << len(pairs)):
        edges = [pairs[i] for i in range(len(pairs)) if mask >> i & 1]
        src = np.array([u for u, _ in edges], np.int32)
        dst = np.array([v for _, v in edges], np.int32)
        rowptr, colidx = oracle.csr_from_edges(6, src, dst)
        assert oracle.triangles(rowptr, colidx) == oracle.brute_force_triangles(6, edges)


def test_golden_per_vertex(golden):
    """Triangles through every vertex against networkx's per-vertex counts."""
    for case in golden:
        rowptr, colidx = csr_of(case)
        total, t = oracle.vertex_triangles(rowptr, colidx)
        assert total == case["triangles"], case["name"]
        assert t.tolist() == case["per_vertex"], case["name"]
        assert int(t.sum()) == 3 * total


def test_random_graphs_per_vertex_brute_force():
    rng = np.random.default_rng(11)
    for n in (7, 9, 12):
        pairs = list(itertools.combinations(range(n), 2))
        for _ in range(200):
            keep = rng.random(len(pairs)) < rng.random()
            edges = [p for p, k in zip(pairs, keep) if k]
            adj = np.zeros((n, n), bool)
            for u, v in edges:
                adj[u, v] = adj[v, u] = True
            expect = [sum(adj[x, y] for x, y in itertools.combinations(np.flatnonzero(adj[u]), 2)) for u in range(n)]
            src = np.array([u for u, _ in edges], np.int32)
            dst = np.array([v for _, v in edges], np.int32)
            rowptr, colidx = oracle.csr_from_edges(n, src, dst)
            assert oracle.vertex_triangles(rowptr, colidx)[1].tolist() == expect


def test_labelled_counts_python_statement(golden):
    """graph.cc:376-391 with the label test, stated in Python on the oriented graph."""
    rng = np.random.default_rng(3)
    for case in golden:
        rowptr, colidx = csr_of(case)
        n = len(rowptr) - 1
        labels = rng.integers(0, 3, n).astype(np.uint8)
        orow, ocol = oracle.orient(rowptr, colidx)
        totals = []
        for label in range(3):
            expect_pe = []
            for u in range(n):
                nu = ocol[orow[u]:orow[u + 1]]
                for v in nu:
                    nv = set(ocol[orow[v]:orow[v + 1]].tolist())
                    expect_pe.append(sum(1 for w in nu.tolist() if w in nv and labels[w] == label))
            total, pe = oracle.labelled(rowptr, colidx, labels, label, per_edge=True)
            assert pe.tolist() == expect_pe, (case["name"], label)
            assert total == sum(expect_pe)
            totals.append(total)
        assert sum(totals) == case["triangles"], case["name"]


def test_random_seven_vertex_graphs():
    rng = np.random.default_rng(7)
    pairs = list(itertools.combinations(range(7), 2))
    for _ in range(3000):
        keep = rng.random(len(pairs)) < rng.random()
        edges = [p for p, k in zip(pairs, keep) if k]
        src = np.array([u for u, _ in edges], np.int32)
        dst = np.array([v for _, v in edges], np.int32)
        rowptr, colidx = oracle.csr_from_edges(7, src, dst)
        assert oracle.triangles(rowptr, colidx) == oracle.brute_force_triangles(7, edges)


def test_relabel_invariance(golden):
    rng = np.random.default_rng(3)
    for case in golden:
        n = case["n"]
        e = np.array(case["edges"], np.int64).reshape(-1, 2)
        perm = rng.permutation(n)
        rowptr, colidx = oracle.csr_from_edges(n, perm[e[:, 0]], perm[e[:, 1]])
        assert oracle.triangles(rowptr, colidx) == case["triangles"]


def test_unsorted_rows_same_dag_after_sort():
    """graph.cc keeps input order; sorting rows first (main.cc:30-31) gives sorted DAG rows."""
    rowptr, colidx = oracle.csr_from_edges(50, *np.random.default_rng(1).integers(0, 50, (2, 400)).astype(np.int32))
    shuffled = colidx.copy()
    rng = np.random.default_rng(2)
    for u in range(50):
        a, b = rowptr[u], rowptr[u + 1]
        shuffled[a:b] = rng.permutation(shuffled[a:b])
    oracle.lib().oracle_sort_neighbors(50, oracle._p(rowptr), oracle._p(shuffled))
    assert np.array_equal(shuffled, colidx)


def test_batch_count_matches_individual(golden):
    graphs = [csr_of(c) for c in golden[:20]]
    vtx_off = np.cumsum([0] + [len(r) - 1 for r, _ in graphs]).astype(np.int64)
    rowptr = [np.zeros(1, np.int64)]
    cols = []
    base = 0
    for r, c in graphs:
        rowptr.append(r[1:] + base)
        cols.append(c)
        base += len(c)
    totals = oracle.batch_count(vtx_off, np.concatenate(rowptr), np.concatenate(cols))
    assert totals.tolist() == [c["triangles"] for c in golden[:20]]


def test_partition_totals_python_statement(golden):
    """The per-PE partial counts (both credit rules) against the PE loops stated in Python."""
    rng = np.random.default_rng(9)
    for case in golden:
        rowptr, colidx = csr_of(case)
        orow, ocol = oracle.orient(rowptr, colidx)
        n = len(orow) - 1
        for k in (1, 2, 3):
            part = rng.integers(0, k, n).astype(np.int64)
            for rule in ("source", "push_pull"):
                total, pt = oracle.partition_totals(orow, ocol, part, k, rule)
                t2, pt2 = oracle.py_partition_totals(orow, ocol, part, k, rule)
                assert pt.tolist() == pt2, (case["name"], k, rule)
                assert total == t2 == case["triangles"]

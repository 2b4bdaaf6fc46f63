"""The oracle pinned to the reference's own code — no GPU needed.

oracle/_ref is the reference's successful_push_pull/graph.cc compiled
unchanged (oracle/build_ref.sh).  Where it is built (the reference tree is
present), the C restatement oracle/tc_oracle.c must give the same oriented
arrays (graph.cc:252-298), the same per-edge and total counts
(graph.cc:376-391 summed as bs_warp_vertex.cuh:13-21) and the same labelled
counts.  Everywhere, the restatement must reproduce the committed fixtures
that the reference's code produced (tests/golden/reference_outputs.json)."""
import numpy as np
import pytest

from oracle import oracle, ref
from reference_fixtures import MAKER, digest, fixtures, golden_inputs, seeded_inputs

needs_ref = pytest.mark.skipif(not ref.available(), reason="reference tree absent: oracle/_ref not built")


def port_orient(rowptr, colidx, sort_neighbors):
    orow, ocol = oracle.orient(rowptr, colidx)
    if sort_neighbors:
        for u in range(len(orow) - 1):
            ocol[orow[u]:orow[u + 1]].sort()
    return orow, ocol


def test_restatement_reproduces_reference_fixtures_golden(golden):
    cases = golden_inputs(golden)
    assert len(cases) >= 30
    for name, rp, col, r in cases:
        orow, ocol = oracle.orient(rp, col)
        assert digest(orow, np.int64) == r["dag_rowptr_sha256"], name
        assert digest(ocol, np.int32) == r["dag_colidx_sha256"], name
        t, pe = oracle.count(orow, ocol, per_edge=True)
        assert t == r["total"], name
        assert digest(pe, np.uint32) == r["per_edge_sha256"], name


def test_restatement_reproduces_reference_fixtures_seeded():
    rec = {r["name"]: r for r in fixtures()["seeded"]}
    for name, (rp, col, lab, classes, srt) in seeded_inputs().items():
        r = rec[name]
        orow, ocol = port_orient(rp, col, srt)
        assert digest(orow, np.int64) == r["dag_rowptr_sha256"], name
        assert digest(ocol, np.int32) == r["dag_colidx_sha256"], name
        if lab is None:
            t, pe = oracle.count(orow, ocol, per_edge=True)
            assert t == r["total"], name
            assert digest(pe, np.uint32) == r["per_edge_sha256"], name
        else:
            for item in r["labelled"]:
                t, pe = oracle.labelled(rp, col, lab, item["label"], per_edge=True)
                assert t == item["total"], (name, item["label"])
                assert digest(pe, np.uint32) == item["per_edge_sha256"], (name, item["label"])


def test_fixtures_cover_long_oriented_rows():
    """One fixture graph has oriented rows longer than 512 entries."""
    assert max(r["max_out_degree"] for r in fixtures()["seeded"]) > 512


@needs_ref
def test_reference_build_matches_restatement_golden(golden):
    for c in golden:
        rp, col = MAKER.golden_csr(c)
        if not ref.accepts(rp):
            continue
        t, pe, orow, ocol = ref.triangles(rp, col, per_edge=True)
        t2, pe2, orow2, ocol2 = oracle.triangles(rp, col, per_edge=True)
        assert t == t2 == c["triangles"], c["name"]
        assert np.array_equal(orow, orow2) and np.array_equal(ocol, ocol2), c["name"]
        assert np.array_equal(pe, pe2), c["name"]


@needs_ref
@pytest.mark.parametrize("seed", range(6))
def test_reference_build_matches_restatement_random(seed):
    """Seeded R-MAT and ER graphs of varied skew, unlabelled and labelled."""
    rng = np.random.default_rng(1000 + seed)
    scale = int(rng.integers(8, 13))
    a = float(rng.uniform(0.45, 0.6))
    b = float(rng.uniform(0.1, 0.25))
    rp, col = MAKER.rmat(scale, 16, seed, a=a, b=b, c=b)
    if not ref.accepts(rp):
        pytest.skip("graph outside what Graph::Graph loads")
    t, pe, orow, ocol = ref.triangles(rp, col, per_edge=True)
    t2, pe2, orow2, ocol2 = oracle.triangles(rp, col, per_edge=True)
    assert t == t2
    assert np.array_equal(orow, orow2) and np.array_equal(ocol, ocol2)
    assert np.array_equal(pe, pe2)
    lab = MAKER.labels_for(len(rp) - 1, 3, seed)
    for label in range(3):
        tl, pel = ref.labelled(rp, col, lab, label, per_edge=True)
        tl2, pel2 = oracle.labelled(rp, col, lab, label, per_edge=True)
        assert tl == tl2 and np.array_equal(pel, pel2), label


@needs_ref
def test_reference_build_unsorted_rows_then_sort():
    """main.cc:19-31 with adj_sorted=0: orientation on the file order, then
    sort_neighbors; the restatement orients in input order and sorts."""
    rp, col = MAKER.er(2000, 20, 11)
    shuffled = MAKER.shuffled_rows(rp, col, 11)
    with ref.RefGraph(rp, shuffled, sort_neighbors=True) as g:
        orow, ocol = g.arrays()
        t, pe = g.count(per_edge=True)
    orow2, ocol2 = port_orient(rp, shuffled, True)
    assert np.array_equal(orow, orow2) and np.array_equal(ocol, ocol2)
    t2, pe2 = oracle.count(orow2, ocol2, per_edge=True)
    assert t == t2 and np.array_equal(pe, pe2)


@pytest.mark.parametrize("kw", [dict(kind="rmat", scale=14, edge_factor=16, seed=3),
                                dict(kind="rmat", scale=12, edge_factor=8, a=0.45, b=0.25, c=0.15, seed=9),
                                dict(kind="er", n=10000, avg_degree=12, seed=1),
                                dict(kind="chung_lu", n=50000, avg_degree=24, gamma=2.1, seed=3)])
def test_oracle_generator_draws_the_engines_samples(kw):
    """CPU-only callers (the timed reference arm) draw the benchmark graph
    with the oracle's generator; it must be the engine's graph."""
    import hetegeneous_parallel_programming_gb300 as tc
    n, s, d = tc.gen_edges_host(tc.GenSpec(**kw))
    k = dict(kw)
    n2, s2, d2 = oracle.gen_edges(k.pop("kind"), **k)
    assert n == n2 and np.array_equal(s, s2) and np.array_equal(d, d2)

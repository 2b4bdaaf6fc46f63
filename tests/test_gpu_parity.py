"""GPU parity: the engine (through the C ABI) against the CPU oracle and the
golden vectors.  Integer results must be bit-exact."""
import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from oracle import oracle

pytestmark = pytest.mark.gpu

ARMS = list(range(tc.TC_NUM_ARMS))


def csr_of(case):
    e = np.array(case["edges"], np.int64).reshape(-1, 2)
    return oracle.csr_from_edges(case["n"], e[:, 0], e[:, 1])


def gen_csr(spec):
    n, s, d = tc.gen_edges_host(spec)
    return oracle.csr_from_edges(n, s, d)


def test_golden_cases_every_arm(engine, golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        for arm in [None] + ARMS:
            total, per_edge, st = engine.count(rowptr, colidx, force_arm=arm, edge_counts=True)
            assert total == case["triangles"], (case["name"], arm)
            assert per_edge.tolist() == case["oriented_per_edge"], (case["name"], arm)


def test_orientation_matches_reference_rule(engine, golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        drow, dcol = engine.orient(rowptr, colidx)
        orow, ocol = oracle.orient(rowptr, colidx)
        assert np.array_equal(drow, orow) and np.array_equal(dcol, ocol), case["name"]


def test_count_dag_matches_reference_solver(engine, golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        orow, ocol = oracle.orient(rowptr, colidx)
        for arm in [None, 0, 3, 5, 9]:
            total, per_edge, _ = engine.count_dag(orow, ocol, force_arm=arm, edge_counts=True)
            ref, ref_pe = oracle.count(orow, ocol, per_edge=True)
            assert total == ref == case["triangles"]
            assert np.array_equal(per_edge, ref_pe)
            total, _, _ = engine.count_dag(orow, ocol, force_arm=arm)
            assert total == ref, (case["name"], arm, "total only")


@pytest.mark.parametrize("spec", [
    tc.GenSpec("er", n=16384, avg_degree=16, seed=0),          # the plain-small workload
    tc.GenSpec("er", n=16384, avg_degree=16, seed=7),
    tc.GenSpec("rmat", scale=14, edge_factor=16, seed=0),
    tc.GenSpec("rmat", scale=16, edge_factor=16, seed=1),
    tc.GenSpec("rmat", scale=16, edge_factor=16, a=0.45, b=0.25, c=0.15, seed=2),
    tc.GenSpec("chung_lu", n=50000, avg_degree=24, gamma=2.1, seed=3),
    tc.GenSpec("rgg", n=8000, avg_degree=40, seed=4),
])
def test_seeded_graphs_bit_exact(engine, spec):
    rowptr, colidx = gen_csr(spec)
    ref_total, ref_pe, orow, ocol = oracle.triangles(rowptr, colidx, per_edge=True)
    for sel, arm in [("fixed", None)] + [("force", a) for a in ARMS]:
        total, per_edge, st = engine.count(rowptr, colidx, selector=sel, force_arm=arm, edge_counts=True)
        assert total == ref_total, (spec, sel, arm)
        assert np.array_equal(per_edge, ref_pe), (spec, sel, arm)
        assert st["m"] == len(ocol)
        # total only (no per-edge output): the arms may take their total-only paths
        total, _, _ = engine.count(rowptr, colidx, selector=sel, force_arm=arm)
        assert total == ref_total, (spec, sel, arm, "total only")
    total, _, _ = engine.count(rowptr, colidx)
    assert total == ref_total


def test_pull_source_blocks_bit_exact(engine):
    """R-MAT scale 20 has more oriented edges than one PULL source block
    (2560 tiles of 4096 edges), so its grouped edges span several blocks."""
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=20, edge_factor=16, seed=4))
    ref_total, ref_pe, _, ocol = oracle.triangles(rowptr, colidx, per_edge=True)
    assert len(ocol) > 2560 * tc.TILE_EDGES
    for sel, arm in [("fixed", None), ("force", 9)]:
        total, per_edge, st = engine.count(rowptr, colidx, selector=sel, force_arm=arm, edge_counts=True)
        assert total == ref_total, (sel, arm)
        assert np.array_equal(per_edge, ref_pe), (sel, arm)
        total, _, _ = engine.count(rowptr, colidx, selector=sel, force_arm=arm)
        assert total == ref_total, (sel, arm, "total only")


def wide_long_lists_graph(k=1100, step=64):
    """Clique on vertex 0 plus k vertices K spread every `step`-th id, and a
    triangle-free k-regular bipartite graph on all other ids.  Every vertex
    has degree k, so ranks follow ids; the first ~74 vertices of K have
    out-lists longer than 1024 entries spanning more than 65536 ids (the PULL
    arm's fallback search).  Triangles: C(k+1, 3), all inside the clique."""
    K = np.arange(1, 1 + k * step, step)[:k]
    n = int(K[-1]) + 2
    fill = np.setdiff1d(np.arange(1, n), K)
    fill = fill[: len(fill) - len(fill) % 2]
    A, B = fill[0::2], fill[1::2]
    clique = np.concatenate([[0], K])
    iu, ju = np.triu_indices(len(clique), 1)
    j = np.arange(k)
    bs = np.repeat(A, k)
    bd = B[(np.repeat(np.arange(len(A)), k) + np.tile(j, len(A))) % len(B)]
    src = np.concatenate([clique[iu], bs]).astype(np.int32)
    dst = np.concatenate([clique[ju], bd]).astype(np.int32)
    return n, src, dst, clique


def test_pull_fallback_wide_long_lists(engine):
    k = 1100
    n, src, dst, clique = wide_long_lists_graph(k)
    rowptr, colidx = engine.csr_from_edges(n, src, dst)
    assert np.all(np.diff(rowptr) == k)
    expect = (k + 1) * k * (k - 1) // 6
    drow, dcol = engine.orient(rowptr, colidx)
    srcs = np.repeat(np.arange(n), np.diff(drow))
    in_clique = np.zeros(n, bool)
    in_clique[clique] = True
    above = np.zeros(n, np.int64)  # clique vertices with a larger id (= higher rank)
    above[clique] = len(clique) - 1 - np.arange(len(clique))
    expect_pe = np.where(in_clique[srcs] & in_clique[dcol], above[dcol], 0).astype(np.uint32)
    for arm in [None, 9]:
        total, pe, st = engine.count(rowptr, colidx, force_arm=arm, edge_counts=True)
        assert total == expect, arm
        assert np.array_equal(pe, expect_pe), arm
        assert engine.count(rowptr, colidx, force_arm=arm)[0] == expect, (arm, "total only")
    total, t, _ = engine.count_vertices(rowptr, colidx)
    assert total == expect
    expect_t = np.zeros(n, np.uint64)
    expect_t[clique] = k * (k - 1) // 2
    assert np.array_equal(t, expect_t)


def test_host_input_uploaded_in_pieces(engine):
    """Host input of >= 2^24 entries is uploaded in pieces behind the
    orientation: a bad id in the last piece or an unsorted row in the first
    is still caught, the call returns cleanly and the ctx counts the intact
    graph exactly afterwards."""
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=20, edge_factor=16, seed=4))
    n = len(rowptr) - 1
    assert len(colidx) >= 1 << 24
    ref = oracle.triangles(rowptr, colidx)
    bad = colidx.copy()
    bad[-1] = n
    with pytest.raises(tc.TCError) as ei:
        engine.count(rowptr, bad)
    assert ei.value.status == 2
    bad = colidx.copy()
    u = int(np.flatnonzero(np.diff(rowptr) >= 2)[0])
    bad[rowptr[u]], bad[rowptr[u] + 1] = bad[rowptr[u] + 1], bad[rowptr[u]]
    with pytest.raises(tc.TCError) as ei:
        engine.count(rowptr, bad)
    assert ei.value.status == 2
    total, pe, st = engine.count(rowptr, colidx, edge_counts=True)
    assert total == ref and int(pe.sum()) == ref
    assert st["h2d_bytes"] == 8 * len(rowptr) + 4 * len(colidx)


def test_pull_chunk_sizes_and_autotune(engine):
    """PULL work-chunk sizes change speed, never counts; the autotuner keeps
    the fastest candidate; the batched path's captured graph follows a change."""
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=16, edge_factor=16, seed=6))
    ref = oracle.triangles(rowptr, colidx)
    old = engine.get_pull_chunks()
    assert old == (512, 128)
    vtx_off = np.array([0, len(rowptr) - 1], np.int64)
    try:
        for item, item_min in ((32, 32), (4096, 64), (512, 128)):
            engine.set_pull_chunks(item, item_min)
            assert engine.count(rowptr, colidx, force_arm=tc.ARM_NAMES.index("pull"))[0] == ref, item
            assert engine.batch_count(vtx_off, rowptr, colidx)[0].tolist() == [ref], item
        best, ms = engine.autotune_pull(rowptr, colidx, candidates=(128, 512, 2048), reps=1)
        assert best in (128, 512, 2048) and sorted(ms) == [128, 512, 2048]
        assert all(t > 0 for t in ms.values()) and ms[best] == min(ms.values())
        assert engine.get_pull_chunks() == (best, max(32, best // 4))
        assert engine.count(rowptr, colidx)[0] == ref
        for bad in ((16, 16), (100, 200), (1 << 17, 64)):
            with pytest.raises(tc.TCError):
                engine.set_pull_chunks(*bad)
        with pytest.raises(tc.TCError):
            engine.autotune_pull(rowptr, colidx, candidates=(8,))
    finally:
        engine.set_pull_chunks(*old)


def test_tuning_changes_speed_not_counts(engine):
    """Every tc_tuning field (PULL chunks, source-block size, dense ratio,
    orientation geometry) leaves totals and per-edge counts bit-exact, on a
    graph whose PULL edges span several source blocks; the autotuner keeps a
    valid setting; out-of-range settings are rejected."""
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=19, edge_factor=16, seed=8))
    ref, ref_pe, _, _ = oracle.triangles(rowptr, colidx, per_edge=True)
    old = engine.get_tuning()
    assert old == {"pull_item": 512, "pull_item_min": 128, "pull_block_tiles": 2560, "pull_dense_num": 1,
                   "pull_dense_den": 1, "orient_blocks_per_sm": 6}
    vtx_off = np.array([0, len(rowptr) - 1], np.int64)
    try:
        for kw in (dict(pull_block_tiles=64), dict(pull_block_tiles=300, pull_dense_num=1, pull_dense_den=8),
                   dict(pull_dense_num=8, pull_dense_den=1, orient_blocks_per_sm=1),
                   dict(orient_blocks_per_sm=64, pull_item=64, pull_item_min=32)):
            engine.set_tuning(**old)
            engine.set_tuning(**kw)
            for sel, arm in (("fixed", None), ("force", tc.ARM_NAMES.index("pull"))):
                total, pe, _ = engine.count(rowptr, colidx, selector=sel, force_arm=arm, edge_counts=True)
                assert total == ref and np.array_equal(pe, ref_pe), (kw, sel)
                assert engine.count(rowptr, colidx, selector=sel, force_arm=arm)[0] == ref, (kw, sel, "total")
            assert engine.batch_count(vtx_off, rowptr, colidx)[0].tolist() == [ref], kw
        engine.set_tuning(**old)
        best, ms, trials = engine.autotune(rowptr, colidx, reps=1)
        assert trials >= 5 and ms > 0 and engine.get_tuning() == best
        assert engine.count(rowptr, colidx)[0] == ref
        for bad in (dict(pull_block_tiles=10), dict(pull_dense_num=0), dict(orient_blocks_per_sm=100),
                    dict(pull_item=16, pull_item_min=16)):
            with pytest.raises(tc.TCError):
                engine.set_tuning(**bad)
        assert engine.get_tuning() == best  # a rejected setting changes nothing
    finally:
        engine.set_tuning(**old)


def test_pull_dense_core(engine):
    """A 3000-vertex core with edge probability 1/2 inside a sparse 200 000-vertex
    graph: the core vertices are the top-ranked hubs and their row suffixes are
    dense, so PULL counts most core edges by ANDing hub bit rows."""
    rng = np.random.default_rng(5)
    n, k = 200000, 3000
    core = rng.choice(n, k, replace=False)
    iu, ju = np.triu_indices(k, 1)
    keep = rng.random(len(iu)) < 0.5
    src = np.concatenate([core[iu[keep]], rng.integers(0, n, 400000)])
    dst = np.concatenate([core[ju[keep]], rng.integers(0, n, 400000)])
    rowptr, colidx = oracle.csr_from_edges(n, src, dst)
    ref, ref_pe, _, _ = oracle.triangles(rowptr, colidx, per_edge=True)
    for arm in (None, tc.ARM_NAMES.index("pull")):
        total, pe, st = engine.count(rowptr, colidx, force_arm=arm, edge_counts=True)
        assert total == ref and np.array_equal(pe, ref_pe), arm
        total, _, _ = engine.count(rowptr, colidx, force_arm=arm)
        assert total == ref, arm
    assert st["tiles_per_arm"]["pull"] > 0


def test_vertex_counts_golden(engine, golden):
    for case in golden:
        rowptr, colidx = csr_of(case)
        total, t, st = engine.count_vertices(rowptr, colidx)
        assert total == case["triangles"], case["name"]
        assert t.tolist() == case["per_vertex"], case["name"]


@pytest.mark.parametrize("spec", [
    tc.GenSpec("er", n=16384, avg_degree=16, seed=0),
    tc.GenSpec("rmat", scale=16, edge_factor=16, seed=1),
    tc.GenSpec("chung_lu", n=50000, avg_degree=24, gamma=2.1, seed=3),
    tc.GenSpec("rgg", n=8000, avg_degree=40, seed=4),
    tc.GenSpec("rmat", scale=20, edge_factor=16, seed=4),  # several PULL source blocks
])
def test_vertex_counts_seeded(engine, spec):
    rowptr, colidx = gen_csr(spec)
    ref_total, ref_t = oracle.vertex_triangles(rowptr, colidx)
    for _ in range(2):  # the top counts start from zero every call
        total, t, _ = engine.count_vertices(rowptr, colidx)
        assert total == ref_total
        assert np.array_equal(t, ref_t)
    local, transitivity = engine.clustering(rowptr, colidx)
    deg = np.diff(rowptr).astype(np.float64)
    pairs = deg * (deg - 1) / 2
    ref_local = np.divide(ref_t.astype(np.float64), pairs, out=np.zeros_like(pairs), where=pairs > 0)
    assert np.allclose(local, ref_local, rtol=0, atol=1e-12)
    assert abs(transitivity - 3 * ref_total / pairs.sum()) < 1e-12


def test_labelled_counts_golden(engine, golden):
    rng = np.random.default_rng(9)
    for case in golden:
        rowptr, colidx = csr_of(case)
        labels = rng.integers(0, 3, len(rowptr) - 1).astype(np.uint8)
        for label in range(3):
            ref, ref_pe = oracle.labelled(rowptr, colidx, labels, label, per_edge=True)
            total, pe, _ = engine.count_labelled(rowptr, colidx, labels, label, edge_counts=True)
            assert total == ref, (case["name"], label)
            assert np.array_equal(pe, ref_pe), (case["name"], label)


@pytest.mark.parametrize("spec", [
    tc.GenSpec("er", n=16384, avg_degree=16, seed=0),
    tc.GenSpec("rmat", scale=16, edge_factor=16, seed=1),
    tc.GenSpec("chung_lu", n=50000, avg_degree=24, gamma=2.1, seed=3),
    tc.GenSpec("rmat", scale=20, edge_factor=16, seed=4),
])
def test_labelled_counts_seeded(engine, spec):
    rowptr, colidx = gen_csr(spec)
    labels = np.random.default_rng(5).integers(0, 4, len(rowptr) - 1).astype(np.uint8)
    ref_all = oracle.triangles(rowptr, colidx)
    totals = []
    for label in range(4):
        ref, ref_pe = oracle.labelled(rowptr, colidx, labels, label, per_edge=True)
        total, pe, _ = engine.count_labelled(rowptr, colidx, labels, label, edge_counts=True)
        assert total == ref and np.array_equal(pe, ref_pe), label
        assert engine.count_labelled(rowptr, colidx, labels, label)[0] == ref, (label, "total only")
        totals.append(total)
    assert sum(totals) == ref_all  # every triangle's highest vertex carries one label


def test_device_generators_match_host(engine):
    import torch
    for spec in [tc.GenSpec("er", n=100000, avg_degree=8, seed=11),
                 tc.GenSpec("rmat", scale=15, edge_factor=8, seed=12),
                 tc.GenSpec("chung_lu", n=60000, avg_degree=12, seed=13)]:
        n, hs, hd = tc.gen_edges_host(spec)
        M = spec.num_samples
        ds = torch.empty(M, dtype=torch.int32, device="cuda")
        dd = torch.empty(M, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        cnt = engine.gen_edges_device(spec, ds.data_ptr(), dd.data_ptr(), M)
        assert cnt == M == len(hs)
        assert np.array_equal(ds.cpu().numpy(), hs) and np.array_equal(dd.cpu().numpy(), hd), spec


def test_device_csr_builder_matches_oracle(engine):
    for spec in [tc.GenSpec("rmat", scale=14, edge_factor=16, seed=5), tc.GenSpec("er", n=3000, avg_degree=30, seed=6)]:
        n, s, d = tc.gen_edges_host(spec)
        r1, c1 = engine.csr_from_edges(n, s, d)
        r2, c2 = oracle.csr_from_edges(n, s, d)
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2)


def test_long_rows_every_sort_class(engine):
    """A clique of 4300 vertices, vertex i with i % 5 pendant neighbours: the
    degree ranks differ from the ids, relabelled rows reach 4299 entries (the
    in-place global row sort), and the answers are analytic: C(k,3)
    triangles; edge u->v inside the clique closes one triangle with every
    clique vertex ranked above v."""
    k = 4300
    iu, ju = np.triu_indices(k, 1)
    pend_owner = np.repeat(np.arange(k), np.arange(k) % 5)
    pend = k + np.arange(len(pend_owner))
    src = np.concatenate([iu, pend_owner]).astype(np.int32)
    dst = np.concatenate([ju, pend]).astype(np.int32)
    n = k + len(pend)
    rowptr, colidx = engine.csr_from_edges(n, src, dst)
    expect = k * (k - 1) * (k - 2) // 6
    deg = np.diff(rowptr)
    rank_order = np.lexsort((np.arange(n), deg))
    rank = np.empty(n, np.int64)
    rank[rank_order] = np.arange(n)
    clique_by_rank = np.sort(rank[:k])  # ranks of the clique vertices, ascending
    above = k - 1 - np.searchsorted(clique_by_rank, rank)  # clique vertices ranked above v
    drow, dcol = engine.orient(rowptr, colidx)
    srcs = np.repeat(np.arange(n), np.diff(drow))
    expect_pe = np.where((srcs < k) & (dcol < k), above[dcol], 0).astype(np.uint32)
    for arm in [None, 0, 1, 8, 9]:
        total, pe, st = engine.count(rowptr, colidx, force_arm=arm, edge_counts=True)
        assert total == expect, arm
        assert np.array_equal(pe, expect_pe), arm
        assert engine.count(rowptr, colidx, force_arm=arm)[0] == expect, (arm, "total only")
    assert int(np.diff(drow).max()) > 4096


def test_wide_rows_of_257_to_4096_entries(engine):
    """Rows of 257..4096 relabelled entries whose ids span more than the
    32768 of a warp bitmap: a circulant graph on G = 36120 vertices (each
    joined to the 130 ids on either side) plus 140 hubs, hub j joined to the
    G vertices j, j + 140, j + 280, ...  Every G vertex then has degree 261,
    so their ranks follow their ids, and each hub (degree 258, ranked below
    them) has a DAG row of 258 entries spanning about 36000 ranks: these
    rows go past the warp bitmap sort to the block sort.  Totals and
    per-edge counts against the oracle."""
    G, half, hubs = 36120, 130, 140
    i = np.repeat(np.arange(G), half)
    j = (i + np.tile(np.arange(1, half + 1), G)) % G
    h = np.repeat(np.arange(hubs), G // hubs)
    t = h + hubs * np.tile(np.arange(G // hubs), hubs)
    src = np.concatenate([i, G + h]).astype(np.int32)
    dst = np.concatenate([j, t]).astype(np.int32)
    rowptr, colidx = engine.csr_from_edges(G + hubs, src, dst)
    ref_total, ref_pe, _, _ = oracle.triangles(rowptr, colidx, per_edge=True)
    deg = np.diff(rowptr)
    assert set(deg[:G]) == {2 * half + 1} and set(deg[G:]) == {G // hubs}
    total, per_edge, _ = engine.count(rowptr, colidx, edge_counts=True)
    assert total == ref_total
    assert np.array_equal(per_edge, ref_pe)
    assert engine.count(rowptr, colidx)[0] == ref_total  # total only: rows without payload


def test_edge_list_entry_path(engine, golden):
    for case in golden:
        e = np.array(case["edges"], np.int64).reshape(-1, 2)
        total, st = engine.count_edges(case["n"], e[:, 0], e[:, 1])
        assert total == case["triangles"], case["name"]
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=14, edge_factor=16, seed=8))
    total, _ = engine.count_edges(n, s, d)
    assert total == oracle.triangles(*oracle.csr_from_edges(n, s, d))


def test_device_pointers_path(engine):
    import torch
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=13, edge_factor=16, seed=3))
    ref, ref_pe, _, _ = oracle.triangles(rowptr, colidx, per_edge=True)
    r = torch.from_numpy(rowptr).cuda()
    c = torch.from_numpy(colidx).cuda()
    out = torch.zeros(len(colidx) // 2, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    total, st = engine.count_device(len(rowptr) - 1, len(colidx), r.data_ptr(), c.data_ptr(),
                                    edge_counts_ptr=out.data_ptr(), edge_capacity=out.numel())
    assert total == ref
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref_pe)


def test_batch_matches_per_graph(engine):
    rng = np.random.default_rng(5)
    graphs = []
    for i in range(120):
        kind = ["er", "rmat", "rgg"][i % 3]
        n = int(np.exp(rng.uniform(np.log(16), np.log(2000))))
        deg = float(rng.uniform(2, 40))
        if kind == "rmat":
            spec = tc.GenSpec("rmat", scale=max(4, int(np.log2(n))), edge_factor=deg / 2, seed=i)
        else:
            spec = tc.GenSpec(kind, n=n, avg_degree=deg, seed=i)
        graphs.append(gen_csr(spec))
    graphs.append(oracle.csr_from_edges(1, np.zeros(0, np.int32), np.zeros(0, np.int32)))  # isolated vertex
    vtx_off = np.cumsum([0] + [len(r) - 1 for r, _ in graphs]).astype(np.int64)
    rows, cols, base = [np.zeros(1, np.int64)], [], 0
    for r, c in graphs:
        rows.append(r[1:] + base)
        cols.append(c)
        base += len(c)
    rowptr, colidx = np.concatenate(rows), np.concatenate(cols)
    ref = oracle.batch_count(vtx_off, rowptr, colidx)
    for arm in [None, 0, 2, 4, 5, 9]:
        totals, st = engine.batch_count(vtx_off, rowptr, colidx, force_arm=arm)
        assert np.array_equal(totals, ref), arm
    # replay of the captured graph gives the same answer
    totals, _ = engine.batch_count(vtx_off, rowptr, colidx)
    totals2, _ = engine.batch_count(vtx_off, rowptr, colidx)
    assert np.array_equal(totals, ref) and np.array_equal(totals2, ref)


def test_batch_local_ids_checked(engine):
    """Batch column ids are local to their graph: an id equal to the graph's
    size (still inside the union) or negative is rejected, with or without
    validation, and the ctx then counts the intact batch."""
    path = oracle.csr_from_edges(4, np.array([0, 1, 2], np.int32), np.array([1, 2, 3], np.int32))
    tri = oracle.csr_from_edges(3, np.array([0, 1, 0], np.int32), np.array([1, 2, 2], np.int32))
    vtx_off = np.array([0, 4, 7], np.int64)
    rowptr = np.concatenate([path[0], tri[0][1:] + len(path[1])]).astype(np.int64)
    colidx = np.concatenate([path[1], tri[1]]).astype(np.int32)
    for bad_id in (4, -1):
        bad = colidx.copy()
        bad[0] = bad_id
        for validate in (True, False):
            with pytest.raises(tc.TCError) as ei:
                engine.batch_count(vtx_off, rowptr, bad, validate=validate)
            assert ei.value.status == 2, (bad_id, validate)
    totals, _ = engine.batch_count(vtx_off, rowptr, colidx)
    assert totals.tolist() == [0, 1]


@pytest.mark.parametrize("rowptr,colidx", [
    ([0, 2, 1, 3], [1, 2, 0]),          # rowptr not monotone
    ([0, 1, 2, 2], [1, 3]),             # id out of range
    ([0, 2, 3, 3], [2, 1, 0]),          # row not ascending
    ([0, 1, 2, 2], [0, 0]),             # self loop
    ([0, 2, 2, 2], [1, 1]),             # duplicate neighbour
    ([0, 1, 2, 5], [1, 0]),             # rowptr[n] != nnz
])
def test_invalid_graphs_rejected(engine, rowptr, colidx):
    n = len(rowptr) - 1
    calls = [lambda: engine.count(np.array(rowptr), np.array(colidx)),
             lambda: engine.count_vertices(np.array(rowptr), np.array(colidx)),
             lambda: engine.count_labelled(np.array(rowptr), np.array(colidx), np.zeros(n, np.uint8), 0)]
    for call in calls:
        with pytest.raises(tc.TCError) as ei:
            call()
        assert ei.value.status == 2
    # the ctx stays usable
    tri = (np.array([0, 2, 4, 6]), np.array([1, 2, 0, 2, 0, 1]))
    assert engine.count(*tri)[0] == 1
    total, t, _ = engine.count_vertices(*tri)
    assert total == 1 and t.tolist() == [1, 1, 1]


def test_labelled_arguments_checked(engine):
    tri = (np.array([0, 2, 4, 6]), np.array([1, 2, 0, 2, 0, 1]))
    with pytest.raises(tc.TCError):
        engine.count_labelled(*tri, np.zeros(3, np.uint8), 256)  # labels are bytes
    with pytest.raises(ValueError):
        engine.count_labelled(*tri, np.zeros(2, np.uint8), 0)    # one label per vertex
    labels = np.array([0, 1, 2], np.uint8)
    # the triangle's highest vertex (rank order: equal degrees, so id 2) carries label 2
    assert [engine.count_labelled(*tri, labels, lab)[0] for lab in range(3)] == [0, 0, 1]


def test_empty_and_tiny(engine):
    with pytest.raises(tc.TCError) as ei:  # a graph needs at least one vertex
        engine.count(np.array([0]), np.zeros(0, np.int32))
    assert ei.value.status == 7
    assert engine.count(np.array([0, 0]), np.zeros(0, np.int32))[0] == 0
    assert engine.count(np.array([0, 0, 0]), np.zeros(0, np.int32))[0] == 0
    assert engine.count(np.array([0, 1, 2]), np.array([1, 0]))[0] == 0


def test_tcsolver_mirror(engine, golden, tmp_path):
    case = next(c for c in golden if c["name"] == "rmat_s10_ef8")
    rowptr, colidx = csr_of(case)
    tc.save_graphminer(str(tmp_path / "graph"), rowptr, colidx)
    g = tc.Graph(str(tmp_path / "graph"), use_dag=True)
    orow, ocol = oracle.orient(rowptr, colidx)
    assert np.array_equal(g.out_rowptr(), orow) and np.array_equal(g.out_colidx(), ocol)
    assert tc.TCSolver(g, 5, 1, 1024) == 5 + case["triangles"]
    dag_only = tc.Graph.from_csr(orow, ocol, oriented=True)
    assert tc.TCSolver(dag_only) == case["triangles"]


def test_cli_matches_reference_usage(golden, tmp_path):
    import subprocess
    from hetegeneous_parallel_programming_gb300 import build
    case = next(c for c in golden if c["name"] == "ba_1500_5")
    rowptr, colidx = csr_of(case)
    tc.save_graphminer(str(tmp_path / "graph"), rowptr, colidx)
    out = subprocess.run([str(build.OUT / "tc_main"), str(tmp_path / "graph"), "1", "1024", "1"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert f"total_num_triangles = {case['triangles']}" in out.stdout


def test_partition_counts_golden(engine, golden):
    """Per-PE partial counts of the partitioned solver, both credit rules."""
    rng = np.random.default_rng(21)
    for case in golden:
        rowptr, colidx = csr_of(case)
        orow, ocol = oracle.orient(rowptr, colidx)
        for k in (1, 3):
            part = rng.integers(0, k, len(orow) - 1).astype(np.int64)
            for rule in ("source", "push_pull"):
                total, pt, _ = engine.count_dag_parts(orow, ocol, part, k, rule=rule)
                ref, ref_pt = oracle.partition_totals(orow, ocol, part, k, rule)
                assert total == ref == case["triangles"], (case["name"], k, rule)
                assert np.array_equal(pt, ref_pt), (case["name"], k, rule)


@pytest.mark.parametrize("k", [8, 5000])  # shared-memory table / global counters
def test_partition_counts_seeded_from_files(engine, tmp_path, metis_writer, k):
    rowptr, colidx = gen_csr(tc.GenSpec("rmat", scale=16, edge_factor=16, seed=3))
    orow, ocol = oracle.orient(rowptr, colidx)
    n = len(orow) - 1
    # contiguous id blocks, as a locality-seeking partitioner would give, with a shuffled tail
    part = (np.arange(n, dtype=np.int64) * k) // n
    tail = np.random.default_rng(k).permutation(n)[: n // 4]
    part[tail] = np.random.default_rng(k + 1).integers(0, k, len(tail))
    prefix = str(tmp_path / "pgraph")
    if k <= 8:  # the file path: write, assemble, count
        metis_writer(prefix, orow, ocol, part, k)
        orow2, ocol2, part2 = tc.assemble_metis(prefix, k)
        assert np.array_equal(orow2, orow) and np.array_equal(ocol2, ocol) and np.array_equal(part2, part)
    for rule in ("source", "push_pull"):
        for arm in (None, 9):
            total, pt, _ = engine.count_dag_parts(orow, ocol, part, k, rule=rule, force_arm=arm)
            ref, ref_pt = oracle.partition_totals(orow, ocol, part, k, rule)
            assert total == ref and np.array_equal(pt, ref_pt), (k, rule, arm)
    total, _, _ = engine.count_dag(orow, ocol)
    assert total == ref


def test_partition_arguments_checked(engine, golden):
    rowptr, colidx = csr_of(golden[0])
    orow, ocol = oracle.orient(rowptr, colidx)
    n = len(orow) - 1
    part = np.zeros(n, np.int64)
    for bad in (-1, 2):
        p = part.copy()
        p[n - 1] = bad
        with pytest.raises(tc.TCError) as ei:
            engine.count_dag_parts(orow, ocol, p, 2)
        assert ei.value.status == 1 and "partition id" in str(ei.value)
    with pytest.raises(tc.TCError):
        engine.count_dag_parts(orow, ocol, part, 0)
    with pytest.raises(ValueError):
        engine.count_dag_parts(orow, ocol, part, 1, rule="owner")
    with pytest.raises(ValueError):
        engine.count_dag_parts(orow, ocol, part[:-1], 1)
    # an unknown rule through the C ABI itself
    import ctypes as C
    from hetegeneous_parallel_programming_gb300 import _ffi
    g = _ffi.Csr(n, len(ocol), orow.ctypes.data, ocol.ctypes.data, 0)
    tot = C.c_uint64(0)
    out = np.zeros(1, np.uint64)
    assert engine._L.tc_count_dag_parts(engine._h, C.byref(g), part.ctypes.data, 1, 7, None, C.byref(tot),
                                        out.ctypes.data, None) == 1
    # the ctx stays usable
    total, pt, _ = engine.count_dag_parts(orow, ocol, part, 1)
    assert total == golden[0]["triangles"] and pt.tolist() == [total]

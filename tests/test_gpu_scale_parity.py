"""GPU parity at the benchmark sizes: the engine against the full CPU oracle
(orientation of graph.cc:252-298, then the merge count of graph.cc:376-391
over every oriented edge, the loop of bs_warp_vertex.cuh:13-21), no row
sampling.  Totals and every uint32 per-edge count must be bit-exact.

  * R-MAT scale 22 and 24, edge factor 16, (a, b, c) = (0.57, 0.19, 0.19),
    seed 0: the plain-at-scale and learned-selector workloads;
  * the 4096-graph mixed batch of the batched workload (seed 1): every
    graph's total;
  * Chung-Lu n = 2^26, average degree 32, gamma 2.1, seed 0: the largest
    single-GPU workload (about 1.06 billion edges, int64 offsets).

The symmetric CSR of each graph is built by the engine's device builder
(test_device_csr_builder_matches_oracle checks it against the oracle's);
the oracle then orients and counts that CSR on the host cores."""
import time

import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from oracle import oracle

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(autouse=True)
def _shipped_selector(engine):
    assert engine.load_shipped_selector()


def build(engine, spec):
    n, s, d = tc.gen_edges_host(spec)
    rowptr, colidx = engine.csr_from_edges(n, s, d)
    return rowptr, colidx


def check_against_full_oracle(engine, spec, selectors=("fixed", "learned")):
    t0 = time.time()
    rowptr, colidx = build(engine, spec)
    t1 = time.time()
    ref_total, ref_pe, orow, ocol = oracle.triangles(rowptr, colidx, per_edge=True)
    t2 = time.time()
    print(f"{spec}: n={len(rowptr) - 1} m={len(ocol)} T={ref_total} build {t1 - t0:.1f}s oracle {t2 - t1:.1f}s")
    for sel in selectors:
        total, pe, st = engine.count(rowptr, colidx, selector=sel, edge_counts=True)
        assert total == ref_total, sel
        assert st["m"] == len(ocol)
        assert np.array_equal(pe, ref_pe), sel
        total, _, _ = engine.count(rowptr, colidx, selector=sel)  # the benchmark's total-only path
        assert total == ref_total, (sel, "total only")
    return ref_total


def test_rmat22_total_and_every_edge(engine):
    check_against_full_oracle(engine, tc.GenSpec("rmat", scale=22, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=0))


def test_rmat24_total_and_every_edge(engine):
    t = check_against_full_oracle(engine, tc.GenSpec("rmat", scale=24, edge_factor=16, a=0.57, b=0.19, c=0.19,
                                                     seed=0))
    assert t == 10281801619  # the benchmark graph's count


def test_batched_4096_graphs_every_total(engine):
    vtx_off, rowptr, colidx = tc.gen_batch_host(4096, seed=1)
    ref = oracle.batch_count(vtx_off, rowptr, colidx)
    for sel in ("fixed", "learned"):
        totals, st = engine.batch_count(vtx_off, rowptr, colidx, selector=sel)
        assert np.array_equal(totals, ref), sel


def test_chung_lu_2p26_total_and_every_edge(engine):
    check_against_full_oracle(engine, tc.GenSpec("chung_lu", n=1 << 26, avg_degree=32, gamma=2.1, seed=0),
                              selectors=("fixed",))

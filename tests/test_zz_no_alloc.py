"""The allocation-free entry point, tc_count_dag_noalloc.

It exists for callers that may not allocate device memory while counting
(applications that own the GPU through their own memory pool, plugins inside
them, latency-bound loops that cannot take cudaMalloc's implicit sync).  The
test calls it through the C ABI on device buffers the test owns and checks
its total and per-edge counts against the allocating entry point
tc_count_dag and the CPU oracle, bit for bit (integer counts), on graphs
whose oriented rows are short (the kernel's hash path) and longer than 512
entries (its per-edge warp search), on two calls in a row: the
second call reuses the static scratch the first one left behind.  This file
sorts last so that a run stopping at the first failure has already run every
other test.
"""
import ctypes as C

import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from hetegeneous_parallel_programming_gb300 import _ffi
from oracle import oracle

pytestmark = pytest.mark.gpu


def _dag(spec):
    if spec == "hubs":  # hubs and a 700-clique: oriented rows of up to 700 entries
        from reference_fixtures import MAKER
        rowptr, colidx = MAKER.hubs(20000, 4)
        return oracle.orient(rowptr, colidx)
    n, s, d = tc.gen_edges_host(spec)
    rowptr, colidx = oracle.csr_from_edges(n, s, d)
    return oracle.orient(rowptr, colidx)


def _noalloc(orow_d, ocol_d, n, m, total_d, counts_d):
    L = _ffi.lib()
    st = L.tc_count_dag_noalloc(0, C.c_void_p(orow_d.data_ptr()), C.c_void_p(ocol_d.data_ptr()), n, m,
                                C.c_void_p(total_d.data_ptr()),
                                C.c_void_p(counts_d.data_ptr()) if counts_d is not None else None, None)
    return st


@pytest.mark.parametrize("spec", [tc.GenSpec("rmat", scale=16, edge_factor=16, seed=3),
                                  tc.GenSpec("er", n=20000, avg_degree=24, seed=4),
                                  "hubs"])
def test_noalloc_matches_allocating_entry_point(spec):
    import torch
    orow, ocol = _dag(spec)
    n, m = len(orow) - 1, len(ocol)
    if spec == "hubs":  # rows longer than 512 entries take the kernel's per-edge warp search
        assert int(np.diff(orow).max()) > 512
    with tc.Engine(0) as eng:
        ref_total, ref_pe, _ = eng.count_dag(orow, ocol, edge_counts=True)
    # the allocating entry point and the CPU oracle agree, so both pin the variant
    o_total, o_pe = oracle.count(orow, ocol, per_edge=True)
    assert ref_total == o_total and np.array_equal(ref_pe, o_pe)
    orow_d = torch.from_numpy(orow).cuda()
    ocol_d = torch.from_numpy(ocol).cuda()
    total_d = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    counts_d = torch.full((m,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        assert _noalloc(orow_d, ocol_d, n, m, total_d, counts_d) == 0, _ffi.lib().tc_last_error(None)
        torch.cuda.synchronize()
        assert int(total_d.item()) == ref_total
        assert np.array_equal(counts_d.cpu().numpy().view(np.uint32), ref_pe)
        counts_d.fill_(-1)
        total_d.fill_(-1)
        torch.cuda.synchronize()
    # without per-edge output
    assert _noalloc(orow_d, ocol_d, n, m, total_d, None) == 0
    torch.cuda.synchronize()
    assert int(total_d.item()) == ref_total


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    orow_d = torch.zeros(2, dtype=torch.int64, device="cuda")
    ocol_d = torch.zeros(1, dtype=torch.int32, device="cuda")
    total_d = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    too_many = (_ffi_max_edges() + 1)
    st = _noalloc(orow_d, ocol_d, 1, too_many, total_d, None)
    assert st == 7  # TC_ERR_UNSUPPORTED, nothing launched
    assert b"static scratch" in _ffi.lib().tc_last_error(None)


def _ffi_max_edges() -> int:
    scratch = 4 << 20          # TC_NOALLOC_SCRATCH_BYTES
    return ((scratch - 256) // 4) * 512

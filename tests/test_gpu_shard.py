"""Row-range shards of the oriented graph (tc_count_dag_range) against the
oracle: contiguous ranges covering all rows give partial counts that add up
to the total, and per-edge counts that concatenate to the whole graph's.
The reference splits rows over GPUs by u % device_count (multigpu.cu:827-843)
and sums the per-device counts on the host (multigpu.cu:930-941); here each
rank counts one range of the replicated graph and one uint64 sum combines."""
import os
import socket

import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from hetegeneous_parallel_programming_gb300 import shard
from oracle import oracle

pytestmark = pytest.mark.gpu


def dag_of(spec):
    n, s, d = tc.gen_edges_host(spec)
    return oracle.orient(*oracle.csr_from_edges(n, s, d))


@pytest.mark.parametrize("spec", [
    tc.GenSpec("er", n=16384, avg_degree=16, seed=0),
    tc.GenSpec("rmat", scale=16, edge_factor=16, seed=1),
    tc.GenSpec("chung_lu", n=50000, avg_degree=24, gamma=2.1, seed=3),
])
def test_ranges_add_up_to_the_whole(engine, spec):
    orow, ocol = dag_of(spec)
    ref, ref_pe = oracle.count(orow, ocol, per_edge=True)
    for parts in (1, 2, 3, 7):
        ranges = shard.balanced_row_ranges(orow, ocol, parts)
        totals, pes = [], []
        for r0, r1 in ranges:
            t, pe, st = engine.count_dag_range(orow, ocol, r0, r1, edge_counts=True)
            assert st["m"] == orow[r1] - orow[r0]
            assert t == int(ref_pe[orow[r0]:orow[r1]].sum(dtype=np.uint64)), (parts, r0, r1)
            t2, _, _ = engine.count_dag_range(orow, ocol, r0, r1)  # total-only path
            assert t2 == t
            totals.append(t)
            pes.append(pe)
        assert sum(totals) == ref, parts
        assert np.array_equal(np.concatenate(pes), ref_pe), parts


def test_range_edge_cases(engine, golden):
    case = next(c for c in golden if c["name"] == "union_K5_K4_wheel6")
    e = np.array(case["edges"], np.int64).reshape(-1, 2)
    orow, ocol = oracle.orient(*oracle.csr_from_edges(case["n"], e[:, 0], e[:, 1]))
    n = len(orow) - 1
    ref, ref_pe = oracle.count(orow, ocol, per_edge=True)
    assert engine.count_dag_range(orow, ocol, 0, n)[0] == ref
    assert engine.count_dag_range(orow, ocol, 3, 3)[0] == 0  # empty range
    for u in range(n):  # one row at a time
        t, pe, _ = engine.count_dag_range(orow, ocol, u, u + 1, edge_counts=True)
        assert t == int(ref_pe[orow[u]:orow[u + 1]].sum()) and np.array_equal(pe, ref_pe[orow[u]:orow[u + 1]])
    for r0, r1 in [(-1, 2), (3, 2), (0, n + 1)]:
        with pytest.raises(tc.TCError) as ei:
            engine.count_dag_range(orow, ocol, r0, r1)
        assert ei.value.status == 1, (r0, r1)


def test_range_on_device_pointers(engine):
    import torch
    orow, ocol = dag_of(tc.GenSpec("rmat", scale=14, edge_factor=16, seed=7))
    ref, ref_pe = oracle.count(orow, ocol, per_edge=True)
    r = torch.from_numpy(orow).cuda()
    c = torch.from_numpy(ocol).cuda()
    torch.cuda.synchronize()
    ranges = shard.balanced_row_ranges(orow, ocol, 4)
    got = [engine.count_dag_range_device(len(orow) - 1, len(ocol), r.data_ptr(), c.data_ptr(), a, b)[0]
           for a, b in ranges]
    assert sum(got) == ref


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, orow, ocol, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r0, r1 = shard.balanced_row_ranges(orow, ocol, world)[rank]
        with tc.Engine(0) as eng:
            local, _, _ = eng.count_dag_range(orow, ocol, r0, r1)
        q.put((rank, local, shard.allreduce_total(local, dist)))
    finally:
        dist.destroy_process_group()


def test_two_processes_sum_their_shards_with_gloo():
    """Two ranks (processes with their own contexts on the one GPU; their
    kernels never wait on each other) count their row ranges and sum over
    gloo."""
    import torch.multiprocessing as mp
    orow, ocol = dag_of(tc.GenSpec("rmat", scale=15, edge_factor=16, seed=2))
    ref = oracle.count(orow, ocol)[0]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, orow, ocol, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1] + out[1][1] == ref
    assert out[0][2] == out[1][2] == ref

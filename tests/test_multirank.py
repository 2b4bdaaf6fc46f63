"""World-size-2 gloo runs on CPU of the multi-rank logic: replica
aggregation (bench) and row-range sharding with one uint64 sum."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from hetegeneous_parallel_programming_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, rowptr, colidx, expect, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        orow, ocol = oracle.orient(rowptr, colidx)
        ranges = shard.balanced_row_ranges(orow, ocol, world)
        r0, r1 = ranges[rank]
        if torch.cuda.is_available():  # the engine counts the shard (tc_count_dag_range)
            import hetegeneous_parallel_programming_gb300 as tc
            with tc.Engine(0) as eng:
                local = eng.count_dag_range(orow, ocol, r0, r1)[0]
        else:  # no GPU here: the oracle stands in for the engine's shard count
            local = int(oracle.lib().oracle_count_rows(len(orow) - 1, oracle._p(orow), oracle._p(ocol), r0, r1, 1,
                                                       None))
        total = shard.allreduce_total(local, dist)
        ms, units = shard.aggregate(10.0 + rank, 100.0 * (rank + 1), dist)
        q.put((rank, total, ms, units, ranges))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_shard_and_aggregate():
    import hetegeneous_parallel_programming_gb300 as tc
    from oracle import oracle
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=12, edge_factor=16, seed=4))
    rowptr, colidx = oracle.csr_from_edges(n, s, d)
    expect = oracle.triangles(rowptr, colidx)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, rowptr, colidx, expect, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, ms, units, ranges in out:
        assert total == expect
        assert ms == 11.0 and units == 300.0
        assert ranges[0][0] == 0 and ranges[-1][1] == n and ranges[0][1] == ranges[1][0]


def test_balanced_ranges_cover_and_balance():
    from oracle import oracle
    import hetegeneous_parallel_programming_gb300 as tc
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=13, edge_factor=16, seed=1))
    orow, ocol = oracle.orient(*oracle.csr_from_edges(n, s, d))
    for parts in (1, 2, 3, 8):
        rr = shard.balanced_row_ranges(orow, ocol, parts)
        assert rr[0][0] == 0 and rr[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rr, rr[1:]))
        parts_total = sum(oracle.lib().oracle_count_rows(n, oracle._p(orow), oracle._p(ocol), a, b, 1, None)
                          for a, b in rr)
        assert parts_total == oracle.count(orow, ocol)[0]


def test_aggregate_without_process_group():
    assert shard.aggregate(3.0, 7.0) == (3.0, 7.0)
    assert shard.allreduce_total(5) == 5

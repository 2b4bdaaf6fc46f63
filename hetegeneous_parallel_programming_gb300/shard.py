"""Multi-rank helpers for the counting path.

The engine runs one graph per GPU, so `bench.py --gpus N` runs N independent
replicas; `aggregate` combines their timings (slowest rank) and units.  For
hosts with several GPUs the path also splits naturally by rows of the
oriented graph: `balanced_row_ranges` cuts the rows into contiguous ranges of
near-equal intersection work, each rank counts its range with the whole
graph replicated read-only, and one uint64 sum (`allreduce_total`) combines
the partial counts — the only exchange the path has.
"""
from __future__ import annotations

import numpy as np


def balanced_row_ranges(dag_rowptr: np.ndarray, dag_colidx: np.ndarray, parts: int) -> list[tuple[int, int]]:
    """Contiguous row ranges [r0, r1) of an oriented graph with near-equal
    work, where a row u costs sum over v in N+(u) of (d+(u) + d+(v))."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    rowptr = np.asarray(dag_rowptr, np.int64)
    n = len(rowptr) - 1
    dplus = np.diff(rowptr)
    src = np.repeat(np.arange(n), dplus)
    edge_cost = dplus[src] + dplus[np.asarray(dag_colidx, np.int64)] if len(dag_colidx) else np.zeros(0, np.int64)
    row_cost = np.zeros(n, np.int64)
    if len(edge_cost):
        np.add.at(row_cost, src, edge_cost)
    row_cost += 1  # every row costs something (its pointer pair)
    cum = np.concatenate([[0], np.cumsum(row_cost)])
    total = cum[-1]
    cuts = [0]
    for p in range(1, parts):
        cuts.append(int(np.searchsorted(cum, total * p / parts, side="left")))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, n))
    return [(int(cuts[i]), int(cuts[i + 1])) for i in range(parts)]


def aggregate(ms_local: float, units_local: float, dist=None, device=None) -> tuple[float, float]:
    """(max ms over ranks, sum of units over ranks); without a process group
    the local values are returned."""
    if dist is None or not dist.is_initialized():
        return ms_local, units_local
    import torch
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    u = torch.tensor([units_local], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def allreduce_total(local_total: int, dist=None, device=None) -> int:
    """Sum of the ranks' partial triangle counts (exact, int64 arithmetic)."""
    if dist is None or not dist.is_initialized():
        return int(local_total)
    import torch
    t = torch.tensor([int(local_total)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())

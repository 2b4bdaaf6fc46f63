import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libtc.so and the oracle once per session (incremental)."""
    from hetegeneous_parallel_programming_gb300 import build as b
    b.build()
    from oracle import oracle
    oracle.lib()


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "triangles.json").read_text())["cases"]


@pytest.fixture(scope="session")
def engine():
    import hetegeneous_parallel_programming_gb300 as tc
    e = tc.Engine(int(os.environ.get("TC_TEST_DEVICE", "0")))
    yield e
    e.close()


def write_metis_parts(prefix, dag_rowptr, dag_colidx, part, num_parts):
    """Partition file sets prefix0 .. prefix{k-1} in the layout of
    PartitionedGraph::metis_write_into_file (graph_partition.cc:501-594):
    partition p keeps an n-row CSR holding only its own vertices' rows
    (global neighbour ids; other rows empty, graph_partition.cc:455-485),
    its vertex list in ascending order and the full part table."""
    import numpy as np
    rowptr = np.asarray(dag_rowptr, np.int64)
    colidx = np.asarray(dag_colidx, np.int32)
    part = np.asarray(part, np.int64)
    n = len(rowptr) - 1
    deg = np.diff(rowptr)
    lists = [np.flatnonzero(part == p).astype(np.int32) for p in range(num_parts)]
    edges = [int(deg[l].sum()) for l in lists]
    for p in range(num_parts):
        own = part == p
        sub_rp = np.concatenate([[0], np.cumsum(np.where(own, deg, 0))]).astype(np.int64)
        sub_col = (np.concatenate([colidx[rowptr[u]:rowptr[u + 1]] for u in lists[p]])
                   if len(lists[p]) else np.zeros(0, np.int32)).astype(np.int32)
        base = f"{prefix}{p}"
        Path(base + ".meta.txt").write_text(
            f"{n}\n{len(lists[p])}\n{edges[p]}\n{max(len(l) for l in lists)}\n{max(edges)}\n{int(deg.max())}\n")
        sub_rp.tofile(base + ".vertex.bin")
        sub_col.tofile(base + ".edge.bin")
        lists[p].tofile(base + ".vertex_list.bin")
        part.tofile(base + ".part.bin")


@pytest.fixture(scope="session")
def metis_writer():
    return write_metis_parts

"""The reference's own CPU graph code, built from its sources — TEST
INFRASTRUCTURE ONLY.

oracle/build_ref.sh compiles the reference's successful_push_pull/graph.cc
unchanged (with oracle/ref_shim/ standing in for the un-vendored GraphMiner
headers) and oracle/ref_driver.cc into oracle/_ref/libtc_ref.so.  This
module feeds it GraphMiner files and reads back:
  - the reference's orientation (Graph::Graph with use_dag, which runs
    Graph::orientation, graph.cc:252-298), and
  - per-edge and total counts from Graph::intersect_num (graph.cc:376-391)
    over every oriented edge, the loop of bs_warp_vertex.cuh:13-21.
It pins oracle/tc_oracle.c and the golden fixtures.  The reference tree is
only present where the fixtures are made; elsewhere available() is False and
the committed fixtures (tests/golden/reference_outputs.json) carry the pin.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_ref" / "libtc_ref.so"
REF_ROOT = Path("/root/reference")
_lib = None


def build() -> bool:
    """Builds oracle/_ref when the reference tree is present; True if built."""
    if not (REF_ROOT / "successful_push_pull" / "graph.cc").exists():
        return False
    subprocess.run(["bash", str(HERE / "build_ref.sh"), str(REF_ROOT)], check=True)
    return SO.exists()


def available() -> bool:
    if SO.exists():
        return True
    return build()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not SO.exists() and not build():
            raise RuntimeError("oracle/_ref is not built (the reference tree is absent)")
        h = C.CDLL(str(SO))
        P, I64 = C.c_void_p, C.c_int64
        h.ref_graph_open.restype = P
        h.ref_graph_open.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int]
        h.ref_graph_close.argtypes = [P]
        for f in ("ref_graph_num_vertices", "ref_graph_num_edges", "ref_graph_max_degree"):
            getattr(h, f).restype = I64
            getattr(h, f).argtypes = [P]
        h.ref_graph_arrays.restype = None
        h.ref_graph_arrays.argtypes = [P, P, P]
        h.ref_graph_count.restype = C.c_uint64
        h.ref_graph_count.argtypes = [P, C.c_int32, I64, I64, I64, P]
        _lib = h
    return _lib


def write_graphminer(prefix: str, rowptr, colidx, labels=None) -> None:
    """GraphMiner files as Graph::Graph reads them (graph.cc:31-55): the
    10-field meta (vid_size 4, eid_size 8, vlabel_size 1), int64 row
    pointers, int32 columns and, with labels, one byte per vertex."""
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    colidx = np.ascontiguousarray(colidx, np.int32)
    n = len(rowptr) - 1
    maxd = int(np.diff(rowptr).max()) if n else 0
    nvc = len(np.unique(labels)) if labels is not None else 0
    Path(prefix + ".meta.txt").write_text(f"{n} {len(colidx)} 4 8 1 0 {maxd} 0 {nvc} 0\n")
    rowptr.tofile(prefix + ".vertex.bin")
    colidx.tofile(prefix + ".edge.bin")
    if labels is not None:
        np.ascontiguousarray(labels, np.uint8).tofile(prefix + ".vlabel.bin")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def accepts(rowptr) -> bool:
    """Graph::Graph asserts 0 < max_degree < n (graph.cc:47): graphs with no
    edge (or a vertex adjacent to all others... never, in a simple graph,
    beyond n-1) are outside what the reference loads."""
    n = len(rowptr) - 1
    return n > 1 and 0 < int(np.diff(rowptr).max()) < n


class RefGraph:
    """A graph opened by the reference's Graph constructor from files."""

    def __init__(self, rowptr, colidx, labels=None, use_dag: bool = True, sort_neighbors: bool = False):
        self._dir = tempfile.TemporaryDirectory(prefix="tc_ref_")
        prefix = str(Path(self._dir.name) / "g" / "graph")
        Path(prefix).parent.mkdir()
        n = len(rowptr) - 1
        lab = np.zeros(n, np.uint8) if labels is None else labels
        write_graphminer(prefix, rowptr, colidx, lab)
        self._h = lib().ref_graph_open(prefix.encode(), int(use_dag), 1, int(sort_neighbors))

    def close(self) -> None:
        if self._h:
            lib().ref_graph_close(self._h)
            self._h = None
        self._dir.cleanup()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def n(self) -> int:
        return int(lib().ref_graph_num_vertices(self._h))

    @property
    def m(self) -> int:
        return int(lib().ref_graph_num_edges(self._h))

    @property
    def max_degree(self) -> int:
        return int(lib().ref_graph_max_degree(self._h))

    def arrays(self):
        rowptr = np.empty(self.n + 1, np.int64)
        colidx = np.empty(max(self.m, 1), np.int32)
        lib().ref_graph_arrays(self._h, _p(rowptr), _p(colidx))
        return rowptr, colidx[:self.m].copy()

    def count(self, label: int = 0, per_edge: bool = False, row_step: int = 1):
        out = np.zeros(max(self.m, 1), np.uint32) if per_edge else None
        t = lib().ref_graph_count(self._h, int(label), 0, self.n, int(row_step), _p(out) if per_edge else None)
        return int(t), (out[:self.m] if per_edge else None)


def triangles(rowptr, colidx, per_edge: bool = False):
    """Reference orientation + count of a symmetric CSR ->
    (total, per-edge counts or None, dag_rowptr, dag_colidx)."""
    with RefGraph(rowptr, colidx) as g:
        orow, ocol = g.arrays()
        t, pe = g.count(per_edge=per_edge)
    return t, pe, orow, ocol


def labelled(rowptr, colidx, labels, label: int, per_edge: bool = False):
    """Reference labelled intersections over the oriented graph."""
    with RefGraph(rowptr, colidx, labels=labels) as g:
        return g.count(label=label, per_edge=per_edge)

"""GB300 exact triangle-counting engine — Python host API over libtc.so.

Mirrors the reference project's host interface for its triangle-counting
path (``Graph`` with GraphMiner CSR loading and ``orientation()``, and
``TCSolver``; reference successful_push_pull/graph.h, multigpu.cu:780) and
exposes the engine's own calls (``Engine.count``, ``Engine.batch_count``,
the learned selector, generators).  Every call goes through the C ABI of
include/tc.h; there is no CPU fallback: without a built libtc.so or without
a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _ffi
from ._ffi import (ARM_NAMES, GEN_CHUNG_LU, GEN_ER, GEN_RGG, GEN_RMAT, SELECT_FIXED, SELECT_FORCE,
                   SELECT_LEARNED, TC_MLP_FEATURES, TC_MLP_PARAM_COUNT, TC_NUM_ARMS, TILE_EDGES)

__all__ = ["TCError", "Engine", "Graph", "TCSolver", "GenSpec", "gen_edges_host", "gen_batch_host",
           "load_vlabels", "save_vlabels",
           "csr_from_edges_host",
           "load_graphminer", "save_graphminer", "load_metis_part", "assemble_metis", "PART_RULES", "check_csr", "ARM_NAMES", "TC_NUM_ARMS", "TC_MLP_FEATURES",
           "TC_MLP_PARAM_COUNT", "TILE_EDGES"]


class TCError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_ffi.STATUS.get(status, status)}: {message}")
        self.status = status


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(st: int, ctx=None) -> None:
    if st != 0:
        msg = _ffi.lib().tc_last_error(ctx)
        raise TCError(st, msg.decode() if msg else "")


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


_SELECTORS = {"fixed": SELECT_FIXED, "learned": SELECT_LEARNED, "force": SELECT_FORCE}


def _opts(selector: str = "fixed", force_arm: Optional[int] = None, validate: bool = True,
          record: bool = False) -> _ffi.Opts:
    o = _ffi.Opts()
    _ffi.lib().tc_opts_default(C.byref(o))
    if force_arm is not None:
        selector = "force"
    if isinstance(force_arm, str):
        force_arm = ARM_NAMES.index(force_arm)
    o.selector = _SELECTORS[selector]
    o.force_arm = int(force_arm or 0)
    o.validate = 1 if validate else 0
    o.record_tile_costs = 1 if record else 0
    return o


# ---- generators ---------------------------------------------------------------------

@dataclass
class GenSpec:
    """A seeded synthetic graph: kind in {'er', 'rmat', 'rgg', 'chung_lu'}."""
    kind: str
    n: int = 0
    scale: int = 0
    avg_degree: float = 16.0
    edge_factor: float = 16.0
    a: float = 0.57
    b: float = 0.19
    c: float = 0.19
    gamma: float = 2.1
    seed: int = 0

    def params(self) -> _ffi.GenParams:
        kinds = {"er": GEN_ER, "rmat": GEN_RMAT, "rgg": GEN_RGG, "chung_lu": GEN_CHUNG_LU}
        p = _ffi.GenParams()
        p.kind = kinds[self.kind]
        p.n = int(self.n)
        p.scale = int(self.scale)
        p.avg_degree = float(self.avg_degree)
        p.edge_factor = float(self.edge_factor)
        p.a, p.b, p.c = float(self.a), float(self.b), float(self.c)
        p.gamma = float(self.gamma)
        p.seed = int(self.seed)
        return p

    @property
    def num_vertices(self) -> int:
        p = self.params()
        return int(_ffi.lib().tc_gen_num_vertices(C.byref(p)))

    @property
    def num_samples(self) -> int:
        p = self.params()
        return int(_ffi.lib().tc_gen_num_samples(C.byref(p)))


def gen_edges_host(spec: GenSpec) -> tuple[int, np.ndarray, np.ndarray]:
    """Edge samples of a seeded generator drawn on the host: (n, src, dst)."""
    L = _ffi.lib()
    p = spec.params()
    cap = int(L.tc_gen_num_samples(C.byref(p)))
    if cap < 0:
        _check(1)
    src = np.empty(max(cap, 1), np.int32)
    dst = np.empty(max(cap, 1), np.int32)
    cnt = C.c_int64(0)
    _check(L.tc_gen_edges_host(C.byref(p), _ptr(src), _ptr(dst), cap, C.byref(cnt)))
    k = cnt.value
    return spec.num_vertices, src[:k], dst[:k]


def csr_from_edges_host(n: int, src: np.ndarray, dst: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Symmetrise + dedup + drop self loops on the host (OpenMP)."""
    L = _ffi.lib()
    src, dst = _i32(src), _i32(dst)
    rp = C.POINTER(C.c_int64)()
    cl = C.POINTER(C.c_int32)()
    nnz = C.c_int64(0)
    _check(L.tc_csr_from_edges_host(int(n), len(src), _ptr(src), _ptr(dst), C.byref(rp), C.byref(cl), C.byref(nnz)))
    try:
        rowptr = np.ctypeslib.as_array(rp, shape=(int(n) + 1,)).copy()
        colidx = np.ctypeslib.as_array(cl, shape=(max(nnz.value, 1),))[:nnz.value].copy()
    finally:
        L.tc_csr_free(C.cast(rp, C.c_void_p), C.cast(cl, C.c_void_p))
    return rowptr, colidx


def gen_batch_host(num_graphs: int = 4096, n_min: int = 64, n_max: int = 16384, deg_min: float = 4.0,
                   deg_max: float = 64.0, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 0):
    """Seeded batch of mixed ER / R-MAT / RGG graphs: (vtx_off, rowptr, colidx) with local ids."""
    L = _ffi.lib()
    spec = _ffi.BatchSpec(int(num_graphs), int(n_min), int(n_max), float(deg_min), float(deg_max), float(a),
                          float(b), float(c), int(seed))
    vtx_off = np.zeros(int(num_graphs) + 1, np.int64)
    rp = C.POINTER(C.c_int64)()
    cl = C.POINTER(C.c_int32)()
    nnz = C.c_int64(0)
    _check(L.tc_gen_batch_host(C.byref(spec), _ptr(vtx_off), C.byref(rp), C.byref(cl), C.byref(nnz)))
    try:
        n = int(vtx_off[-1])
        rowptr = np.ctypeslib.as_array(rp, shape=(n + 1,)).copy()
        colidx = np.ctypeslib.as_array(cl, shape=(max(nnz.value, 1),))[:nnz.value].copy()
    finally:
        L.tc_csr_free(C.cast(rp, C.c_void_p), C.cast(cl, C.c_void_p))
    return vtx_off, rowptr, colidx


def load_graphminer(prefix: str) -> tuple[np.ndarray, np.ndarray]:
    L = _ffi.lib()
    n, nnz, md = C.c_int64(0), C.c_int64(0), C.c_int64(0)
    rp = C.POINTER(C.c_int64)()
    cl = C.POINTER(C.c_int32)()
    _check(L.tc_load_graphminer(str(prefix).encode(), C.byref(n), C.byref(nnz), C.byref(rp), C.byref(cl),
                                C.byref(md)))
    try:
        rowptr = np.ctypeslib.as_array(rp, shape=(n.value + 1,)).copy()
        colidx = np.ctypeslib.as_array(cl, shape=(max(nnz.value, 1),))[:nnz.value].copy()
    finally:
        L.tc_csr_free(C.cast(rp, C.c_void_p), C.cast(cl, C.c_void_p))
    return rowptr, colidx


def save_graphminer(prefix: str, rowptr: np.ndarray, colidx: np.ndarray) -> None:
    rowptr, colidx = _i64(rowptr), _i32(colidx)
    _check(_ffi.lib().tc_save_graphminer(str(prefix).encode(), len(rowptr) - 1, len(colidx), _ptr(rowptr),
                                         _ptr(colidx)))


def load_vlabels(prefix: str, n: int) -> np.ndarray:
    """Vertex labels of a GraphMiner graph (prefix.vlabel.bin, one byte per vertex)."""
    out = np.zeros(int(n), np.uint8)
    _check(_ffi.lib().tc_load_vlabels(str(prefix).encode(), int(n), _ptr(out)))
    return out


def save_vlabels(prefix: str, labels: np.ndarray) -> None:
    labels = np.ascontiguousarray(labels, np.uint8)
    _check(_ffi.lib().tc_save_vlabels(str(prefix).encode(), len(labels), _ptr(labels)))


def load_metis_part(prefix: str) -> dict:
    """One partition file set of a METIS-partitioned graph (prefix e.g.
    "<graph dir>/metis/pgraph0"): sizes from the meta file and the arrays
    rowptr [n+1], colidx [nnz], vertex_list [n_real], part [n]
    (graph_partition.cc:501-594 writes them, graph.cc:16-58 reads them)."""
    L = _ffi.lib()
    mp = _ffi.MetisPart()
    _check(L.tc_load_metis_part(str(prefix).encode(), C.byref(mp)))
    try:
        out = {k: int(getattr(mp, k)) for k in ("n", "n_real", "nnz", "max_subg_nv", "max_subg_ne", "max_degree")}
        out["rowptr"] = np.ctypeslib.as_array(mp.rowptr, shape=(mp.n + 1,)).copy()
        out["colidx"] = np.ctypeslib.as_array(mp.colidx, shape=(max(mp.nnz, 1),))[:mp.nnz].copy()
        out["vertex_list"] = np.ctypeslib.as_array(mp.vertex_list, shape=(max(mp.n_real, 1),))[:mp.n_real].copy()
        out["part"] = np.ctypeslib.as_array(mp.part, shape=(mp.n,)).copy()
    finally:
        L.tc_metis_part_free(C.byref(mp))
    return out


def assemble_metis(prefix: str, num_parts: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The whole oriented graph from partition file sets prefix0 ..
    prefix{num_parts-1}: (rowptr, colidx, part), each row taken from the
    partition that owns it, after the consistency checks of tc_assemble_metis."""
    L = _ffi.lib()
    n, nnz = C.c_int64(0), C.c_int64(0)
    rp = C.POINTER(C.c_int64)()
    cl = C.POINTER(C.c_int32)()
    pt = C.POINTER(C.c_int64)()
    _check(L.tc_assemble_metis(str(prefix).encode(), int(num_parts), C.byref(n), C.byref(nnz), C.byref(rp),
                               C.byref(cl), C.byref(pt)))
    try:
        rowptr = np.ctypeslib.as_array(rp, shape=(n.value + 1,)).copy()
        colidx = np.ctypeslib.as_array(cl, shape=(max(nnz.value, 1),))[:nnz.value].copy()
        part = np.ctypeslib.as_array(pt, shape=(n.value,)).copy()
    finally:
        L.tc_csr_free(C.cast(rp, C.c_void_p), C.cast(cl, C.c_void_p))
        L.tc_host_free(C.cast(pt, C.c_void_p))
    return rowptr, colidx, part


PART_RULES = {"source": _ffi.PART_BY_SOURCE, "push_pull": _ffi.PART_PUSH_PULL}


def check_csr(rowptr: np.ndarray, colidx: np.ndarray, sorted_simple: bool = True) -> None:
    rowptr, colidx = _i64(rowptr), _i32(colidx)
    _check(_ffi.lib().tc_check_csr_host(len(rowptr) - 1, len(colidx), _ptr(rowptr), _ptr(colidx),
                                        1 if sorted_simple else 0))


# ---- engine ----------------------------------------------------------------------------

class Engine:
    """A tc_ctx: one CUDA stream and a grow-only device arena on one GPU."""

    def __init__(self, device: int = 0):
        self._L = _ffi.lib()
        h = C.c_void_p()
        _check(self._L.tc_ctx_create(int(device), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.tc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _chk(self, st: int) -> None:
        _check(st, self._h)

    def sync(self) -> None:
        self._chk(self._L.tc_ctx_sync(self._h))

    @property
    def stream(self) -> int:
        """cudaStream_t of this engine (wrap with torch.cuda.ExternalStream to time it)."""
        return int(self._L.tc_ctx_stream(self._h) or 0)

    def arena_bytes(self) -> int:
        return int(self._L.tc_ctx_arena_bytes(self._h))

    # -- hot path (host arrays) --
    def count(self, rowptr, colidx, *, selector: str = "fixed", force_arm=None, edge_counts: bool = False,
              validate: bool = True):
        """Orient + count a symmetric CSR.  Returns (total, per-edge counts or None, stats dict)."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        out = np.empty(max(len(colidx), 1), np.uint32) if edge_counts else None
        self._chk(self._L.tc_count(self._h, C.byref(g), C.byref(o), C.byref(tot), _ptr(out),
                                   len(colidx) if edge_counts else 0, C.byref(st)))
        if out is not None:
            out = out[:st.m]
        return int(tot.value), out, st.as_dict()

    def count_vertices(self, rowptr, colidx, *, validate: bool = True):
        """Triangles through every vertex of a symmetric CSR: (total, uint64 counts per vertex, stats dict)."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts("fixed", None, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        out = np.zeros(max(len(rowptr) - 1, 1), np.uint64)
        self._chk(self._L.tc_count_vertices(self._h, C.byref(g), C.byref(o), C.byref(tot), _ptr(out), C.byref(st)))
        return int(tot.value), out[:len(rowptr) - 1], st.as_dict()

    def count_labelled(self, rowptr, colidx, labels, label: int, *, edge_counts: bool = False,
                       validate: bool = True):
        """Common out-neighbours carrying `label` over every oriented edge (the reference's labelled
        intersection on the degree-ordered DAG): (total, per-edge counts or None, stats dict)."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        labels = np.ascontiguousarray(labels, np.uint8)
        if len(labels) != len(rowptr) - 1:
            raise ValueError("one label per vertex")
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts("fixed", None, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        out = np.empty(max(len(colidx), 1), np.uint32) if edge_counts else None
        self._chk(self._L.tc_count_labelled(self._h, C.byref(g), _ptr(labels), int(label), C.byref(o), C.byref(tot),
                                            _ptr(out), len(colidx) if edge_counts else 0, C.byref(st)))
        if out is not None:
            out = out[:st.m]
        return int(tot.value), out, st.as_dict()

    def clustering(self, rowptr, colidx, *, validate: bool = True):
        """Local clustering coefficient of every vertex, 2 t(u) / (deg(u) (deg(u) - 1)) (0 below degree 2),
        and the global transitivity 3 T / (number of paths of length 2)."""
        total, t, _ = self.count_vertices(rowptr, colidx, validate=validate)
        deg = np.diff(np.asarray(rowptr, np.int64)).astype(np.float64)
        pairs = deg * (deg - 1) / 2
        local = np.divide(t.astype(np.float64), pairs, out=np.zeros_like(pairs), where=pairs > 0)
        wedges = pairs.sum()
        return local, (3.0 * total / wedges if wedges > 0 else 0.0)

    def count_dag(self, rowptr, colidx, *, selector: str = "fixed", force_arm=None, edge_counts: bool = False,
                  validate: bool = True):
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        out = np.empty(max(len(colidx), 1), np.uint32) if edge_counts else None
        self._chk(self._L.tc_count_dag(self._h, C.byref(g), C.byref(o), C.byref(tot), _ptr(out),
                                       len(colidx) if edge_counts else 0, C.byref(st)))
        if out is not None:
            out = out[:len(colidx)]
        return int(tot.value), out, st.as_dict()

    def count_dag_range(self, rowptr, colidx, row_begin: int, row_end: int, *, selector: str = "fixed",
                        force_arm=None, edge_counts: bool = False, validate: bool = True):
        """One shard of count_dag: the edges of rows [row_begin, row_end) of an
        oriented graph, counted against the whole graph.  Returns (partial
        total, per-edge counts of the range or None, stats dict)."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        rb, re = int(row_begin), int(row_end)
        width = int(rowptr[re] - rowptr[rb]) if 0 <= rb <= re < len(rowptr) else 0
        out = np.empty(max(width, 1), np.uint32) if edge_counts else None
        self._chk(self._L.tc_count_dag_range(self._h, C.byref(g), rb, re, C.byref(o), C.byref(tot), _ptr(out),
                                             width if edge_counts else 0, C.byref(st)))
        if out is not None:
            out = out[:width]
        return int(tot.value), out, st.as_dict()

    def count_dag_range_device(self, n: int, nnz: int, rowptr_ptr: int, colidx_ptr: int, row_begin: int,
                               row_end: int, *, selector: str = "fixed", validate: bool = True):
        """count_dag_range on a device-resident oriented graph: (partial total, stats dict)."""
        g = _ffi.Csr(int(n), int(nnz), int(rowptr_ptr), int(colidx_ptr), 1)
        o = _opts(selector, None, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count_dag_range(self._h, C.byref(g), int(row_begin), int(row_end), C.byref(o),
                                             C.byref(tot), None, 0, C.byref(st)))
        return int(tot.value), st.as_dict()

    def count_dag_parts(self, rowptr, colidx, part, num_parts: int, *, rule: str = "source",
                        selector: str = "fixed", force_arm=None, validate: bool = True):
        """Per-partition partial counts of an oriented graph split by part
        (int64[n]): (total, part_totals uint64[num_parts], stats).  rule
        "source" credits edge u->v to part[u]; "push_pull" follows the
        reference's push/pull split (a cross-partition edge with
        d+(u) < d+(v) is credited to part[v])."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        part = np.ascontiguousarray(part, np.int64)
        if len(part) != len(rowptr) - 1:
            raise ValueError(f"part holds {len(part)} entries, the graph {len(rowptr) - 1} vertices")
        if rule not in PART_RULES:
            raise ValueError(f"rule must be one of {sorted(PART_RULES)}")
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        out = np.zeros(max(int(num_parts), 1), np.uint64)
        st = _ffi.Stats()
        self._chk(self._L.tc_count_dag_parts(self._h, C.byref(g), _ptr(part), int(num_parts), PART_RULES[rule],
                                             C.byref(o), C.byref(tot), _ptr(out), C.byref(st)))
        return int(tot.value), out[:int(num_parts)], st.as_dict()

    def count_edges(self, n: int, src, dst, *, selector: str = "fixed", force_arm=None):
        """Triangles of an undirected edge list (duplicates and self loops allowed)."""
        src, dst = _i32(src), _i32(dst)
        o = _opts(selector, force_arm, True)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count_edges(self._h, int(n), len(src), _ptr(src), _ptr(dst), 0, C.byref(o),
                                         C.byref(tot), C.byref(st)))
        return int(tot.value), st.as_dict()

    def orient(self, rowptr, colidx):
        """Reference orientation (graph.cc:252-298) on the GPU: (dag_rowptr, dag_colidx)."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        drow = np.empty(len(rowptr), np.int64)
        dcol = np.empty(max(len(colidx), 1), np.int32)
        m = C.c_int64(0)
        self._chk(self._L.tc_orient(self._h, C.byref(g), _ptr(drow), _ptr(dcol), len(colidx), C.byref(m)))
        return drow, dcol[:m.value]

    # -- hot path (device pointers, e.g. torch tensors' data_ptr()) --
    def count_device(self, n: int, nnz: int, rowptr_ptr: int, colidx_ptr: int, *, selector: str = "fixed",
                     force_arm=None, edge_counts_ptr: int = 0, edge_capacity: int = 0, validate: bool = True):
        g = _ffi.Csr(int(n), int(nnz), int(rowptr_ptr), int(colidx_ptr), 1)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count(self._h, C.byref(g), C.byref(o), C.byref(tot),
                                   C.c_void_p(edge_counts_ptr) if edge_counts_ptr else None, int(edge_capacity),
                                   C.byref(st)))
        return int(tot.value), st.as_dict()

    def count_vertices_device(self, n: int, nnz: int, rowptr_ptr: int, colidx_ptr: int, vertex_counts_ptr: int, *,
                              validate: bool = True):
        """Per-vertex triangle counts of a device-resident CSR into a device uint64 buffer of n entries."""
        g = _ffi.Csr(int(n), int(nnz), int(rowptr_ptr), int(colidx_ptr), 1)
        o = _opts("fixed", None, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count_vertices(self._h, C.byref(g), C.byref(o), C.byref(tot),
                                            C.c_void_p(vertex_counts_ptr), C.byref(st)))
        return int(tot.value), st.as_dict()

    def count_labelled_device(self, n: int, nnz: int, rowptr_ptr: int, colidx_ptr: int, labels_ptr: int, label: int,
                              *, validate: bool = True):
        """Labelled count of a device-resident CSR with device labels (n bytes): (total, stats dict)."""
        g = _ffi.Csr(int(n), int(nnz), int(rowptr_ptr), int(colidx_ptr), 1)
        o = _opts("fixed", None, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count_labelled(self._h, C.byref(g), C.c_void_p(labels_ptr), int(label), C.byref(o),
                                            C.byref(tot), None, 0, C.byref(st)))
        return int(tot.value), st.as_dict()

    def count_host_ptr(self, n: int, nnz: int, rowptr_ptr: int, colidx_ptr: int, *, selector: str = "fixed",
                       force_arm=None, validate: bool = True):
        """Like count() but on caller-owned host buffers (e.g. pinned memory)."""
        g = _ffi.Csr(int(n), int(nnz), int(rowptr_ptr), int(colidx_ptr), 0)
        o = _opts(selector, force_arm, validate)
        tot = C.c_uint64(0)
        st = _ffi.Stats()
        self._chk(self._L.tc_count(self._h, C.byref(g), C.byref(o), C.byref(tot), None, 0, C.byref(st)))
        return int(tot.value), st.as_dict()

    # -- batched --
    def batch_count(self, vtx_off, rowptr, colidx, *, selector: str = "fixed", force_arm=None,
                    validate: bool = True):
        vtx_off, rowptr, colidx = _i64(vtx_off), _i64(rowptr), _i32(colidx)
        b = _ffi.Batch(len(vtx_off) - 1, _ptr(vtx_off).value, _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, force_arm, validate)
        totals = np.zeros(len(vtx_off) - 1, np.uint64)
        st = _ffi.Stats()
        self._chk(self._L.tc_batch_count(self._h, C.byref(b), C.byref(o), _ptr(totals), C.byref(st)))
        return totals, st.as_dict()

    def batch_count_device(self, num_graphs: int, vtx_off_ptr: int, rowptr_ptr: int, colidx_ptr: int, *,
                           selector: str = "fixed", force_arm=None, validate: bool = True):
        b = _ffi.Batch(int(num_graphs), int(vtx_off_ptr), int(rowptr_ptr), int(colidx_ptr), 1)
        o = _opts(selector, force_arm, validate)
        totals = np.zeros(int(num_graphs), np.uint64)
        st = _ffi.Stats()
        self._chk(self._L.tc_batch_count(self._h, C.byref(b), C.byref(o), _ptr(totals), C.byref(st)))
        return totals, st.as_dict()

    # -- learned selector --
    def tile_profile(self, rowptr, colidx):
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        cap = len(colidx) // TILE_EDGES + 2
        feats = np.zeros((cap, TC_MLP_FEATURES), np.float32)
        costs = np.zeros((cap, TC_NUM_ARMS), np.float32)
        t = C.c_int64(0)
        self._chk(self._L.tc_tile_profile(self._h, C.byref(g), _ptr(feats), _ptr(costs), cap, C.byref(t)))
        return feats[:t.value].copy(), costs[:t.value].copy()

    def plan_arms(self, rowptr, colidx, *, selector: str = "fixed") -> np.ndarray:
        """The arm the selector picks for every 4096-edge tile."""
        rowptr, colidx = _i64(rowptr), _i32(colidx)
        g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector)
        cap = len(colidx) // TILE_EDGES + 2
        arms = np.zeros(cap, np.int32)
        t = C.c_int64(0)
        self._chk(self._L.tc_plan_arms(self._h, C.byref(g), C.byref(o), _ptr(arms), cap, C.byref(t)))
        return arms[:t.value].copy()

    def train_selector(self, features, costs, *, epochs: int = 60, lr: float = 2e-3, weight_decay: float = 0.0,
                       seed: int = 0) -> float:
        features = np.ascontiguousarray(features, np.float32)
        costs = np.ascontiguousarray(costs, np.float32)
        loss = C.c_float(0)
        self._chk(self._L.tc_selector_train(self._h, _ptr(features), _ptr(costs), len(features), int(epochs),
                                            float(lr), float(weight_decay), int(seed), C.byref(loss)))
        return float(loss.value)

    def set_pull_chunks(self, item: int, item_min: int) -> None:
        """PULL work-chunk sizes (largest, smallest) used by later calls."""
        self._chk(self._L.tc_set_pull_chunks(self._h, int(item), int(item_min)))

    def get_pull_chunks(self) -> tuple[int, int]:
        a, b = C.c_int32(0), C.c_int32(0)
        self._chk(self._L.tc_get_pull_chunks(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def autotune_pull(self, rowptr, colidx, candidates=(256, 512, 1024, 2048), reps: int = 3, *,
                      selector: str = "fixed", on_device_n: int = 0):
        """Counts the graph with each candidate PULL chunk size and keeps the
        fastest in this engine: (best, {candidate: ms}).  rowptr/colidx are
        host arrays, or device pointers when on_device_n (the vertex count)
        is given, with colidx then the entry count paired as (ptr, nnz)."""
        if on_device_n:
            (rp_ptr, cl_ptr, nnz) = rowptr, colidx[0], colidx[1]
            g = _ffi.Csr(int(on_device_n), int(nnz), int(rp_ptr), int(cl_ptr), 1)
        else:
            rowptr, colidx = _i64(rowptr), _i32(colidx)
            g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        cands = np.ascontiguousarray(candidates, np.int32)
        ms = np.zeros(len(cands), np.float32)
        best = C.c_int32(0)
        o = _opts(selector, None, True)
        self._chk(self._L.tc_autotune_pull(self._h, C.byref(g), C.byref(o), _ptr(cands), len(cands), int(reps),
                                           ms.ctypes.data_as(C.POINTER(C.c_float)), C.byref(best)))
        return int(best.value), {int(c): float(t) for c, t in zip(cands, ms)}

    def get_tuning(self) -> dict:
        """The engine's run-time tuning (tc_tuning) as a dict."""
        t = _ffi.Tuning()
        self._chk(self._L.tc_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw) -> None:
        """Changes fields of the run-time tuning (tc_tuning); the rest keep their values."""
        t = _ffi.Tuning(**self.get_tuning())
        for k, v in kw.items():
            if k not in dict(_ffi.Tuning._fields_):
                raise ValueError(f"unknown tuning field {k}")
            setattr(t, k, int(v))
        self._chk(self._L.tc_set_tuning(self._h, C.byref(t)))

    def autotune(self, rowptr, colidx, reps: int = 2, *, selector: str = "fixed", on_device_n: int = 0):
        """Coordinate-descent autotuner over the PULL chunk size, source-block
        size, dense ratio and orientation geometry (tc_autotune); keeps the
        fastest setting in this engine.  Returns (tuning dict, ms, trials).
        rowptr/colidx are host arrays, or device pointers when on_device_n
        (the vertex count) is given, with colidx then paired as (ptr, nnz)."""
        if on_device_n:
            (rp_ptr, cl_ptr, nnz) = rowptr, colidx[0], colidx[1]
            g = _ffi.Csr(int(on_device_n), int(nnz), int(rp_ptr), int(cl_ptr), 1)
        else:
            rowptr, colidx = _i64(rowptr), _i32(colidx)
            g = _ffi.Csr(len(rowptr) - 1, len(colidx), _ptr(rowptr).value, _ptr(colidx).value, 0)
        o = _opts(selector, None, True)
        t = _ffi.Tuning()
        ms = C.c_float(0)
        trials = C.c_int32(0)
        self._chk(self._L.tc_autotune(self._h, C.byref(g), C.byref(o), int(reps), C.byref(t), C.byref(ms),
                                      C.byref(trials)))
        return t.as_dict(), float(ms.value), int(trials.value)

    def l2_bandwidth(self, nbytes: int = 64 << 20, passes: int = 128) -> float:
        """L2 read ceiling in GB/s: one kernel streams an L2-resident buffer
        `passes` times with L1-bypassing 16-byte loads (tc_l2_bandwidth)."""
        g = C.c_double(0.0)
        self._chk(self._L.tc_l2_bandwidth(self._h, int(nbytes), int(passes), C.byref(g)))
        return float(g.value)

    def set_selector_weights(self, params) -> None:
        params = np.ascontiguousarray(params, np.float32)
        self._chk(self._L.tc_selector_set_weights(self._h, _ptr(params), len(params)))

    def load_shipped_selector(self) -> bool:
        """Loads the shipped MLP cost-model weights (data/selector_mlp.npz)
        and their switching margin for selector="learned"; False when the
        file is absent or holds weights for another arm set."""
        path = Path(__file__).resolve().parent / "data" / "selector_mlp.npz"
        if not path.exists():
            return False
        z = np.load(path)
        w = z["params"].astype(np.float32)
        if w.size != TC_MLP_PARAM_COUNT:
            return False
        self.set_selector_weights(w)
        self.set_selector_margin(float(z["margin"]) if "margin" in z.files else 0.0)
        return True

    def set_selector_margin(self, margin: float) -> None:
        """log2-cost gain the learned selector needs to leave the fixed rule's arm."""
        self._chk(self._L.tc_selector_set_margin(self._h, float(margin)))

    def get_selector_weights(self) -> np.ndarray:
        out = np.zeros(TC_MLP_PARAM_COUNT, np.float32)
        self._chk(self._L.tc_selector_get_weights(self._h, _ptr(out), len(out)))
        return out

    def selector_predict(self, features) -> np.ndarray:
        features = np.ascontiguousarray(features, np.float32)
        out = np.zeros((len(features), TC_NUM_ARMS), np.float32)
        self._chk(self._L.tc_selector_predict(self._h, _ptr(features), len(features), _ptr(out)))
        return out

    def selector_grad(self, params, features, targets):
        params = np.ascontiguousarray(params, np.float32)
        features = np.ascontiguousarray(features, np.float32)
        targets = np.ascontiguousarray(targets, np.float32)
        loss = C.c_float(0)
        grad = np.zeros(TC_MLP_PARAM_COUNT, np.float32)
        self._chk(self._L.tc_selector_grad(self._h, _ptr(params), _ptr(features), _ptr(targets), len(features),
                                           C.byref(loss), _ptr(grad)))
        return float(loss.value), grad

    # -- graph construction on the device --
    def csr_from_edges(self, n: int, src, dst):
        src, dst = _i32(src), _i32(dst)
        rowptr = np.empty(int(n) + 1, np.int64)
        cap = 2 * len(src)
        colidx = np.empty(max(cap, 1), np.int32)
        nnz = C.c_int64(0)
        self._chk(self._L.tc_csr_from_edges(self._h, int(n), len(src), _ptr(src), _ptr(dst), 0, _ptr(rowptr),
                                            _ptr(colidx), cap, C.byref(nnz)))
        return rowptr, colidx[:nnz.value]

    def csr_from_edges_device(self, n: int, m: int, src_ptr: int, dst_ptr: int, rowptr_ptr: int,
                              colidx_ptr: int, capacity: int) -> int:
        nnz = C.c_int64(0)
        self._chk(self._L.tc_csr_from_edges(self._h, int(n), int(m), C.c_void_p(src_ptr), C.c_void_p(dst_ptr), 1,
                                            C.c_void_p(rowptr_ptr), C.c_void_p(colidx_ptr), int(capacity),
                                            C.byref(nnz)))
        return int(nnz.value)

    def gen_edges_device(self, spec: GenSpec, src_ptr: int, dst_ptr: int, capacity: int) -> int:
        p = spec.params()
        cnt = C.c_int64(0)
        self._chk(self._L.tc_gen_edges_device(self._h, C.byref(p), C.c_void_p(src_ptr), C.c_void_p(dst_ptr),
                                              int(capacity), C.byref(cnt)))
        return int(cnt.value)


_shared_engine: Optional[Engine] = None


def _engine() -> Engine:
    global _shared_engine
    if _shared_engine is None:
        _shared_engine = Engine(0)
    return _shared_engine


# ---- reference-shaped host interface ----------------------------------------------------

class Graph:
    """GraphMiner CSR graph (reference successful_push_pull/graph.h:14-188).

    ``Graph(prefix, use_dag)`` loads prefix.meta.txt/.vertex.bin/.edge.bin and
    orients when use_dag (the orientation runs on the GPU and keeps exactly
    the reference's edges and neighbour order).  ``Graph.from_csr`` wraps
    arrays already in memory.
    """

    def __init__(self, prefix: Optional[str] = None, use_dag: bool = False, directed: bool = False):
        self._sym: Optional[tuple[np.ndarray, np.ndarray]] = None
        self.oriented = False
        self.directed = directed
        if prefix is None:
            self.vertices = np.zeros(1, np.int64)
            self.edges = np.zeros(0, np.int32)
            return
        self.vertices, self.edges = load_graphminer(prefix)
        if use_dag:
            if directed:
                raise ValueError("orientation needs an undirected graph")
            self.orientation()

    @classmethod
    def from_csr(cls, rowptr, colidx, oriented: bool = False) -> "Graph":
        g = cls()
        g.vertices, g.edges = _i64(rowptr), _i32(colidx)
        g.oriented = oriented
        return g

    def V(self) -> int:
        return len(self.vertices) - 1

    def E(self) -> int:
        return len(self.edges)

    num_vertices = size = V
    num_edges = sizeEdges = E

    def get_degree(self, v: int) -> int:
        return int(self.vertices[v + 1] - self.vertices[v])

    out_degree = get_degree

    def edge_begin(self, v: int) -> int:
        return int(self.vertices[v])

    def edge_end(self, v: int) -> int:
        return int(self.vertices[v + 1])

    def N(self, v: int, i: Optional[int] = None):
        row = self.edges[self.vertices[v]:self.vertices[v + 1]]
        return row if i is None else int(row[i])

    def out_rowptr(self) -> np.ndarray:
        return self.vertices

    def out_colidx(self) -> np.ndarray:
        return self.edges

    def get_max_degree(self) -> int:
        return int(np.max(np.diff(self.vertices))) if self.V() > 0 else 0

    def is_oriented(self) -> bool:
        return self.oriented

    def orientation(self) -> None:
        if self.oriented:
            return
        drow, dcol = _engine().orient(self.vertices, self.edges)
        self._sym = (self.vertices, self.edges)
        self.vertices, self.edges = drow, dcol
        self.oriented = True

    def sort_neighbors(self) -> None:
        for v in range(self.V()):
            a, b = self.vertices[v], self.vertices[v + 1]
            self.edges[a:b] = np.sort(self.edges[a:b])

    def print_meta_data(self) -> None:
        print(f"|V|: {self.V()}, |E|: {self.E()}, Max Degree: {self.get_max_degree()}"
              + (" (oriented)" if self.oriented else ""))


def TCSolver(g: Graph, total: int = 0, n_gpu: int = 1, chunk_size: int = 1024) -> int:
    """Reference TCSolver(Graph&, uint64_t& total, n_gpu, chunk_size): returns total + count.

    chunk_size is ignored (as in the reference); every n_gpu counts on device 0.
    """
    eng = _engine()
    if g._sym is not None:
        t, _, _ = eng.count(*g._sym)
    elif g.oriented:
        t, _, _ = eng.count_dag(g.vertices, g.edges)
    else:
        t, _, _ = eng.count(g.vertices, g.edges)
    return int(total) + t

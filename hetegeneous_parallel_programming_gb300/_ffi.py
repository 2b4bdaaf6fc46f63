"""ctypes declarations of the C ABI in include/tc.h (libtc.so).

The library is loaded from the package's in-tree ``_build/`` directory only;
there is no fallback implementation, so a missing build raises at import of
the first call.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libtc.so"

TC_NUM_ARMS = 10
TC_MLP_FEATURES = 16
TC_MLP_HIDDEN = 64
TC_MLP_PARAM_COUNT = (TC_MLP_FEATURES * TC_MLP_HIDDEN + TC_MLP_HIDDEN + TC_MLP_HIDDEN * TC_MLP_HIDDEN +
                      TC_MLP_HIDDEN + TC_MLP_HIDDEN * TC_NUM_ARMS + TC_NUM_ARMS)
TILE_EDGES = 4096

ARM_NAMES = ["bsearch4", "bsearch32", "merge8", "merge32", "hash", "bitmap", "gallop4", "mpath2", "flat", "pull"]

SELECT_FIXED, SELECT_LEARNED, SELECT_FORCE = 0, 1, 2
GEN_ER, GEN_RMAT, GEN_RGG, GEN_CHUNG_LU = 0, 1, 2, 3

STATUS = {0: "ok", 1: "invalid argument", 2: "invalid graph", 3: "CUDA error", 4: "out of memory",
          5: "I/O error", 6: "device wait timed out", 7: "unsupported size", 8: "no CUDA device"}


class Csr(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("rowptr", C.c_void_p), ("colidx", C.c_void_p),
                ("on_device", C.c_int32)]


class Opts(C.Structure):
    _fields_ = [("selector", C.c_int32), ("force_arm", C.c_int32), ("record_tile_costs", C.c_int32),
                ("validate", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("ms_h2d", C.c_float), ("ms_validate", C.c_float), ("ms_orient", C.c_float),
                ("ms_plan", C.c_float), ("ms_count", C.c_float), ("ms_scatter", C.c_float),
                ("ms_d2h", C.c_float), ("ms_total", C.c_float), ("m", C.c_int64), ("tiles", C.c_int64),
                ("tiles_per_arm", C.c_int64 * TC_NUM_ARMS), ("kernel_launches", C.c_int64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("ms_arm", C.c_float * TC_NUM_ARMS),
                ("alg_bytes_arm", C.c_uint64 * TC_NUM_ARMS), ("alg_bytes", C.c_uint64),
                ("ms_pull_kernel", C.c_float), ("pull_edges", C.c_uint64)]

    _PER_ARM = ("tiles_per_arm", "ms_arm", "alg_bytes_arm")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in self._PER_ARM}
        for k in self._PER_ARM:
            arr = getattr(self, k)
            d[k] = {ARM_NAMES[i]: (float(arr[i]) if k == "ms_arm" else int(arr[i])) for i in range(TC_NUM_ARMS)}
        return d


class MetisPart(C.Structure):
    _fields_ = [("n", C.c_int64), ("n_real", C.c_int64), ("nnz", C.c_int64), ("max_subg_nv", C.c_int64),
                ("max_subg_ne", C.c_int64), ("max_degree", C.c_int64), ("rowptr", C.POINTER(C.c_int64)),
                ("colidx", C.POINTER(C.c_int32)), ("vertex_list", C.POINTER(C.c_int32)),
                ("part", C.POINTER(C.c_int64))]


PART_BY_SOURCE, PART_PUSH_PULL = 0, 1


class Batch(C.Structure):
    _fields_ = [("num_graphs", C.c_int64), ("vtx_off", C.c_void_p), ("rowptr", C.c_void_p),
                ("colidx", C.c_void_p), ("on_device", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("pull_item", C.c_int32), ("pull_item_min", C.c_int32), ("pull_block_tiles", C.c_int32),
                ("pull_dense_num", C.c_int32), ("pull_dense_den", C.c_int32), ("orient_blocks_per_sm", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class BatchSpec(C.Structure):
    _fields_ = [("num_graphs", C.c_int64), ("n_min", C.c_int64), ("n_max", C.c_int64), ("deg_min", C.c_double),
                ("deg_max", C.c_double), ("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("seed", C.c_uint64)]


class GenParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n", C.c_int64), ("scale", C.c_int32), ("avg_degree", C.c_double),
                ("edge_factor", C.c_double), ("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("gamma", C.c_double), ("seed", C.c_uint64)]


P = C.c_void_p
I64, I32, U64 = C.c_int64, C.c_int32, C.c_uint64
PI64 = C.POINTER(C.c_int64)
PU64 = C.POINTER(C.c_uint64)
PF = C.POINTER(C.c_float)

_SIGS = {
    "tc_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "tc_ctx_destroy": (None, [P]),
    "tc_last_error": (C.c_char_p, [P]),
    "tc_status_str": (C.c_char_p, [C.c_int]),
    "tc_opts_default": (None, [C.POINTER(Opts)]),
    "tc_ctx_arena_bytes": (I64, [P]),
    "tc_ctx_sync": (C.c_int, [P]),
    "tc_ctx_stream": (P, [P]),
    "tc_orient": (C.c_int, [P, C.POINTER(Csr), P, P, I64, PI64]),
    "tc_count": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), PU64, P, I64, C.POINTER(Stats)]),
    "tc_count_dag": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), PU64, P, I64, C.POINTER(Stats)]),
    "tc_count_dag_range": (C.c_int, [P, C.POINTER(Csr), I64, I64, C.POINTER(Opts), PU64, P, I64,
                                     C.POINTER(Stats)]),
    "tc_count_vertices": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), PU64, P, C.POINTER(Stats)]),
    "tc_count_labelled": (C.c_int, [P, C.POINTER(Csr), P, I32, C.POINTER(Opts), PU64, P, I64, C.POINTER(Stats)]),
    "tc_batch_count": (C.c_int, [P, C.POINTER(Batch), C.POINTER(Opts), P, C.POINTER(Stats)]),
    "tc_count_dag_noalloc": (C.c_int, [C.c_int, P, P, I64, I64, P, P, P]),
    "tc_l2_bandwidth": (C.c_int, [P, I64, I32, C.POINTER(C.c_double)]),
    "tc_set_pull_chunks": (C.c_int, [P, I32, I32]),
    "tc_get_pull_chunks": (C.c_int, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tc_autotune_pull": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), P, I32, I32, PF, C.POINTER(C.c_int32)]),
    "tc_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "tc_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "tc_autotune": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), I32, C.POINTER(Tuning), PF, C.POINTER(C.c_int32)]),
    "tc_count_dag_parts": (C.c_int, [P, C.POINTER(Csr), P, I32, I32, C.POINTER(Opts), PU64, P, C.POINTER(Stats)]),
    "tc_count_edges": (C.c_int, [P, I64, I64, P, P, I32, C.POINTER(Opts), PU64, C.POINTER(Stats)]),
    "tc_tile_profile": (C.c_int, [P, C.POINTER(Csr), P, P, I64, PI64]),
    "tc_plan_arms": (C.c_int, [P, C.POINTER(Csr), C.POINTER(Opts), P, I64, PI64]),
    "tc_selector_train": (C.c_int, [P, P, P, I64, I32, C.c_float, C.c_float, U64, PF]),
    "tc_selector_set_margin": (C.c_int, [P, C.c_float]),
    "tc_selector_set_weights": (C.c_int, [P, P, I64]),
    "tc_selector_get_weights": (C.c_int, [P, P, I64]),
    "tc_selector_predict": (C.c_int, [P, P, I64, P]),
    "tc_selector_grad": (C.c_int, [P, P, P, P, I64, PF, P]),
    "tc_csr_from_edges": (C.c_int, [P, I64, I64, P, P, I32, P, P, I64, PI64]),
    "tc_gen_num_samples": (I64, [C.POINTER(GenParams)]),
    "tc_gen_num_vertices": (I64, [C.POINTER(GenParams)]),
    "tc_gen_edges_host": (C.c_int, [C.POINTER(GenParams), P, P, I64, PI64]),
    "tc_gen_edges_device": (C.c_int, [P, C.POINTER(GenParams), P, P, I64, PI64]),
    "tc_gen_batch_host": (C.c_int, [C.POINTER(BatchSpec), P, C.POINTER(PI64), C.POINTER(C.POINTER(C.c_int32)),
                                    PI64]),
    "tc_csr_from_edges_host": (C.c_int, [I64, I64, P, P, C.POINTER(PI64), C.POINTER(C.POINTER(C.c_int32)), PI64]),
    "tc_load_graphminer": (C.c_int, [C.c_char_p, PI64, PI64, C.POINTER(PI64), C.POINTER(C.POINTER(C.c_int32)),
                                     PI64]),
    "tc_save_graphminer": (C.c_int, [C.c_char_p, I64, I64, P, P]),
    "tc_load_vlabels": (C.c_int, [C.c_char_p, I64, P]),
    "tc_save_vlabels": (C.c_int, [C.c_char_p, I64, P]),
    "tc_csr_free": (None, [P, P]),
    "tc_load_metis_part": (C.c_int, [C.c_char_p, C.POINTER(MetisPart)]),
    "tc_metis_part_free": (None, [C.POINTER(MetisPart)]),
    "tc_assemble_metis": (C.c_int, [C.c_char_p, I32, PI64, PI64, C.POINTER(PI64), C.POINTER(C.POINTER(C.c_int32)),
                                    C.POINTER(PI64)]),
    "tc_host_free": (None, [P]),
    "tc_check_csr_host": (C.c_int, [I64, I64, P, P, I32]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """The loaded libtc.so; raises if the extension has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"libtc.so is not built ({LIB_PATH}); run "
                                   "`python -c 'import __graft_entry__ as g; g.build()'` first")
            h = C.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGS.items():
                f = getattr(h, name)
                f.restype = res
                f.argtypes = args
            _lib = h
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)

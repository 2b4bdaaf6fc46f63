"""Builds baseline/_build/libtc_refgpu.so (the reference-kernel restatement)
and loads it.  Baseline only: the engine never links it."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "warp_vertex_ref.cu"
SO = HERE / "_build" / "libtc_refgpu.so"
_lib = None


def build() -> Path:
    SO.parent.mkdir(exist_ok=True)
    if not SO.exists() or SO.stat().st_mtime < SRC.stat().st_mtime:
        tmp = SO.with_suffix(".tmp")
        subprocess.run(["nvcc", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-shared",
                        "-Xcompiler", "-fPIC", "-o", str(tmp), str(SRC)], check=True)
        tmp.replace(SO)
    return SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        h = C.CDLL(str(SO))
        h.tc_ref_warp_vertex.restype = C.c_int
        h.tc_ref_warp_vertex.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_float)]
        _lib = h
    return _lib


def count(rowptr_ptr: int, col_ptr: int, n: int) -> tuple[int, float]:
    """(total, kernel ms) of the reference-style kernel on a device DAG."""
    t = C.c_uint64(0)
    ms = C.c_float(0)
    err = lib().tc_ref_warp_vertex(C.c_void_p(rowptr_ptr), C.c_void_p(col_ptr), int(n), C.byref(t), C.byref(ms))
    if err != 0:
        raise RuntimeError(f"reference-style kernel failed with CUDA error {err}")
    return int(t.value), float(ms.value)

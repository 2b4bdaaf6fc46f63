"""Build recipe for libtc.so (the engine) — nvcc for sm_103a, g++ for host C++.

Every translation unit is compiled in parallel into ``_build/`` next to this
file and linked into ``_build/libtc.so``.  Objects are rebuilt only when a
source or header is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = PKG.parent / "include"
LIB = OUT / "libtc.so"

CU_SOURCES = ["radix_sort.cu", "orient.cu", "count.cu", "capi.cu", "build_graph.cu", "mlp.cu", "batch.cu", "noalloc.cu"]
CPP_SOURCES = ["host_graph.cpp", "solver.cpp"]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + sorted(
        INCLUDE.glob("*.hpp"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in _headers()) or \
        Path(__file__).stat().st_mtime > t


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for name in CU_SOURCES:
        src = CSRC / name
        obj = OUT / (name + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_verbose:
            cmd = [nvcc, ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "--expt-relaxed-constexpr", *common,
                   "-c", str(src), "-o", str(obj)]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for name in CPP_SOURCES:
        src = CSRC / name
        obj = OUT / (name + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["g++", "-fPIC", "-fopenmp", "-Wall", "-Wno-unknown-pragmas", *common,
                         "-I/usr/local/cuda/include", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        futs = [ex.submit(_run, j) for j in jobs]
        for f in futs:
            f.result()
    if jobs or not LIB.exists():
        tmp = OUT / "libtc.so.tmp"
        _run([nvcc, ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(tmp), *map(str, objs), "-lgomp"])
        os.replace(tmp, LIB)
    cli = OUT / "tc_main"
    main_src = CSRC / "tc_main.cpp"
    if not cli.exists() or cli.stat().st_mtime < LIB.stat().st_mtime or main_src.stat().st_mtime > cli.stat().st_mtime:
        _run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", "-o", str(cli), str(main_src), f"-L{OUT}", "-ltc",
              f"-Wl,-rpath,{OUT}", "-fopenmp"])
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)

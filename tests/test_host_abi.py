"""Host-side logic and the C ABI surface (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import hetegeneous_parallel_programming_gb300 as tc
from hetegeneous_parallel_programming_gb300 import _ffi
from oracle import oracle

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "tc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    L = _ffi.lib()
    names = declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(_ffi.exported_symbols())


def test_cpp_mirror_symbols_exported():
    so = C.CDLL(str(_ffi.LIB_PATH))
    assert hasattr(so, "_Z8TCSolverR5GraphRmii")  # TCSolver(Graph&, unsigned long&, int, int)


def test_status_strings():
    L = _ffi.lib()
    for s in range(9):
        assert L.tc_status_str(s).decode() == _ffi.STATUS[s]


def test_no_device_is_reported_not_crashed():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(tc.TCError) as ei:
        tc.Engine(0)
    assert ei.value.status == 8


@pytest.mark.parametrize("spec", [
    tc.GenSpec("er", n=5000, avg_degree=12, seed=3),
    tc.GenSpec("rmat", scale=12, edge_factor=8, seed=1),
    tc.GenSpec("chung_lu", n=4000, avg_degree=10, gamma=2.1, seed=5),
    tc.GenSpec("rgg", n=3000, avg_degree=9, seed=2),
])
def test_host_generators_deterministic_and_in_range(spec):
    n, s1, d1 = tc.gen_edges_host(spec)
    n2, s2, d2 = tc.gen_edges_host(spec)
    assert n == n2 and np.array_equal(s1, s2) and np.array_equal(d1, d2)
    assert len(s1) > 0 and s1.min() >= 0 and d1.min() >= 0 and s1.max() < n and d1.max() < n
    other = tc.GenSpec(**{**spec.__dict__, "seed": spec.seed + 1})
    _, s3, _ = tc.gen_edges_host(other)
    assert not (len(s3) == len(s1) and np.array_equal(s3, s1))


def test_rmat_degree_skew():
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=14, edge_factor=16, seed=0))
    deg = np.bincount(np.concatenate([s, d]), minlength=n)
    assert deg[0] > 50 * deg.mean()  # vertex 0 collects quadrant a at every level


def test_rgg_average_degree_close_to_target():
    n, s, d = tc.gen_edges_host(tc.GenSpec("rgg", n=20000, avg_degree=20, seed=4))
    assert 0.85 * 20 < 2 * len(s) / n < 1.05 * 20


def test_host_csr_builder_matches_oracle():
    n, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=11, edge_factor=16, seed=9))
    r1, c1 = tc.csr_from_edges_host(n, s, d)
    r2, c2 = oracle.csr_from_edges(n, s, d)
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    tc.check_csr(r1, c1, sorted_simple=True)


def test_graphminer_round_trip(tmp_path):
    n, s, d = tc.gen_edges_host(tc.GenSpec("er", n=700, avg_degree=6, seed=1))
    r, c = tc.csr_from_edges_host(n, s, d)
    tc.save_graphminer(str(tmp_path / "g"), r, c)
    meta = (tmp_path / "g.meta.txt").read_text().split()
    assert meta[:4] == [str(n), str(len(c)), "4", "8"]
    assert int(meta[6]) == int(np.diff(r).max())
    r2, c2 = tc.load_graphminer(str(tmp_path / "g"))
    assert np.array_equal(r, r2) and np.array_equal(c, c2)
    g = tc.Graph(str(tmp_path / "g"))
    assert g.V() == n and g.E() == len(c) and g.get_degree(3) == r[4] - r[3]


def test_vertex_labels_round_trip(tmp_path):
    n, s, d = tc.gen_edges_host(tc.GenSpec("er", n=300, avg_degree=5, seed=2))
    r, c = tc.csr_from_edges_host(n, s, d)
    tc.save_graphminer(str(tmp_path / "g"), r, c)
    labels = np.random.default_rng(1).integers(0, 5, n).astype(np.uint8)
    tc.save_vlabels(str(tmp_path / "g"), labels)
    meta = (tmp_path / "g.meta.txt").read_text().split()
    assert meta[4] == "1" and int(meta[8]) == int(labels.max()) + 1  # label size, vertex classes
    assert np.array_equal(tc.load_vlabels(str(tmp_path / "g"), n), labels)
    r2, c2 = tc.load_graphminer(str(tmp_path / "g"))  # the graph still loads
    assert np.array_equal(r, r2) and np.array_equal(c, c2)
    with pytest.raises(tc.TCError):
        tc.load_vlabels(str(tmp_path / "g"), n + 1)  # wrong length


def test_graphminer_malformed_files(tmp_path):
    r = np.array([0, 1, 2], np.int64)
    c = np.array([1, 0], np.int32)
    tc.save_graphminer(str(tmp_path / "ok"), r, c)
    # truncated edge file
    (tmp_path / "ok.edge.bin").write_bytes(c.tobytes()[:4])
    with pytest.raises(tc.TCError) as ei:
        tc.load_graphminer(str(tmp_path / "ok"))
    assert ei.value.status == 5
    # missing files
    with pytest.raises(tc.TCError) as ei:
        tc.load_graphminer(str(tmp_path / "nope"))
    assert ei.value.status == 5
    # wrong id width
    tc.save_graphminer(str(tmp_path / "w"), r, c)
    meta = (tmp_path / "w.meta.txt").read_text().replace("4 8", "8 8", 1)
    (tmp_path / "w.meta.txt").write_text(meta)
    with pytest.raises(tc.TCError) as ei:
        tc.load_graphminer(str(tmp_path / "w"))
    assert ei.value.status == 7
    # out-of-range id in an otherwise well-formed file
    (tmp_path / "bad.meta.txt").write_text("2\n2\n4 8 1 4\n1\n0\n0\n0\n")
    (tmp_path / "bad.vertex.bin").write_bytes(r.tobytes())
    (tmp_path / "bad.edge.bin").write_bytes(np.array([1, 5], np.int32).tobytes())
    with pytest.raises(tc.TCError) as ei:
        tc.load_graphminer(str(tmp_path / "bad"))
    assert ei.value.status == 2


@pytest.mark.parametrize("rowptr,colidx,why", [
    ([0, 2, 1, 3], [1, 2, 0], "monotone"),
    ([0, 1, 2, 2], [1, 3], "range"),
    ([0, 2, 3, 3], [1, 1, 0], "ascending"),
    ([0, 1, 2, 2], [0, 0], "self loop"),
    ([1, 1, 2, 2], [0, 0], "rowptr"),
])
def test_check_csr_rejects(rowptr, colidx, why):
    with pytest.raises(tc.TCError) as ei:
        tc.check_csr(np.array(rowptr), np.array(colidx), sorted_simple=True)
    assert ei.value.status == 2


def _partitioned_dag(seed=4, n=600, k=4):
    nn, s, d = tc.gen_edges_host(tc.GenSpec("rmat", scale=9, edge_factor=8, seed=seed))
    r, c = oracle.csr_from_edges(nn, s, d)
    orow, ocol = oracle.orient(r, c)
    part = np.random.default_rng(seed).integers(0, k, len(orow) - 1).astype(np.int64)
    return orow, ocol, part


def test_metis_parts_load_and_assemble(tmp_path, metis_writer):
    orow, ocol, part = _partitioned_dag()
    (tmp_path / "metis").mkdir()
    prefix = str(tmp_path / "metis" / "pgraph")
    metis_writer(prefix, orow, ocol, part, 4)
    deg = np.diff(orow)
    for p in range(4):
        mp = tc.load_metis_part(prefix + str(p))
        own = np.flatnonzero(part == p)
        assert mp["n"] == len(orow) - 1 and mp["n_real"] == len(own)
        assert mp["nnz"] == int(deg[own].sum()) and mp["max_degree"] == int(deg.max())
        assert np.array_equal(mp["vertex_list"], own) and np.array_equal(mp["part"], part)
        sub_deg = np.diff(mp["rowptr"])
        assert np.array_equal(sub_deg, np.where(part == p, deg, 0))
    r, c, pt = tc.assemble_metis(prefix, 4)
    assert np.array_equal(r, orow) and np.array_equal(c, ocol) and np.array_equal(pt, part)


def test_metis_parts_inconsistent_rejected(tmp_path, metis_writer):
    orow, ocol, part = _partitioned_dag(seed=5, k=3)
    prefix = str(tmp_path / "pgraph")
    metis_writer(prefix, orow, ocol, part, 3)
    with pytest.raises(tc.TCError) as ei:  # a fourth file set does not exist
        tc.assemble_metis(prefix, 4)
    assert ei.value.status == 5
    # a part table that differs between file sets
    other = part.copy()
    other[0] = (other[0] + 1) % 3
    other.tofile(prefix + "1.part.bin")
    with pytest.raises(tc.TCError) as ei:
        tc.assemble_metis(prefix, 3)
    assert ei.value.status == 2
    # partition ids outside [0, num_parts): the same files read as two partitions
    metis_writer(prefix, orow, ocol, part, 3)
    with pytest.raises(tc.TCError) as ei:
        tc.assemble_metis(prefix, 2)
    assert ei.value.status == 2
    # a vertex list that misses a vertex
    vl = np.fromfile(prefix + "0.vertex_list.bin", np.int32)
    vl[-1] = vl[0]
    vl.tofile(prefix + "0.vertex_list.bin")
    with pytest.raises(tc.TCError) as ei:
        tc.assemble_metis(prefix, 3)
    assert ei.value.status == 2
    # a row with entries in a partition that does not own it
    metis_writer(prefix, orow, ocol, part, 3)
    deg = np.diff(orow)
    u = int(np.flatnonzero((part != 0) & (deg > 0))[0])
    rows = (part == 0) | (np.arange(len(deg)) == u)
    np.concatenate([[0], np.cumsum(np.where(rows, deg, 0))]).astype(np.int64).tofile(prefix + "0.vertex.bin")
    np.concatenate([ocol[orow[v]:orow[v + 1]] for v in np.flatnonzero(rows)]).astype(np.int32).tofile(
        prefix + "0.edge.bin")
    meta = (tmp_path / "pgraph0.meta.txt").read_text().split()
    meta[2] = str(int(deg[rows].sum()))
    (tmp_path / "pgraph0.meta.txt").write_text("\n".join(meta) + "\n")
    assert tc.load_metis_part(prefix + "0")["nnz"] == int(deg[rows].sum())  # the file set itself reads
    with pytest.raises(tc.TCError) as ei:
        tc.assemble_metis(prefix, 3)
    assert ei.value.status == 2 and "outside partition 0 hold entries" in str(ei.value)
    # a truncated vertex list against its meta file
    metis_writer(prefix, orow, ocol, part, 3)
    vl = np.fromfile(prefix + "2.vertex_list.bin", np.int32)
    vl[:-1].tofile(prefix + "2.vertex_list.bin")
    with pytest.raises(tc.TCError) as ei:
        tc.load_metis_part(prefix + "2")
    assert ei.value.status == 5


def test_selector_batch_union_is_the_disjoint_union():
    """The trainer's small-graph batch union: a valid simple symmetric CSR in
    global ids whose triangles are the batch's per-graph triangles."""
    from hetegeneous_parallel_programming_gb300.train_selector import batch_union
    rowptr, colidx = batch_union(24, seed=5)
    tc.check_csr(rowptr, colidx, sorted_simple=True)
    vtx_off, lrow, lcol = tc.gen_batch_host(24, seed=5)
    assert np.array_equal(rowptr, lrow)
    assert oracle.triangles(rowptr, colidx) == int(oracle.batch_count(vtx_off, lrow, lcol).sum())


def _bench(args, env=None):
    import json
    import os
    import subprocess
    import sys
    e = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    e.update(env or {})
    r = subprocess.run([sys.executable, str(ROOT / "bench.py")] + args, env=e, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    return [json.loads(ln) for ln in lines]


def test_bench_reference_arm_line():
    """The reference arm times the oracle's orientation + merge count on the
    host cores and prints one line with the engine arm's metric and unit."""
    (line,) = _bench(["--impl", "reference", "--workload", "er16k", "--steps", "3", "--warmup", "3",
                      "--ref-step-seconds", "0.2"])
    assert line["impl"] == "reference"
    assert line["unit"] == "GTEPS" and line["higher_is_better"] is True and line["value"] > 0
    assert (line["n_gpus"], line["steps"], line["warmup"]) == (1, 3, 3)
    assert line["config"]["n"] == 16384 and line["config"]["workload"].startswith("Erdos-Renyi")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert "graph.cc:252-298" in cb["sample"] and "graph.cc:376-391" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["vs_baseline"] is None


def test_bench_reference_arm_other_ranks_silent():
    """Under torchrun only rank 0 runs the CPU path; the others exit 0 with no line."""
    assert _bench(["--impl", "reference", "--workload", "er16k", "--steps", "1", "--warmup", "1"],
                  env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_bench_reference_arm_does_not_load_the_engine():
    """The reference arm draws its graph with the oracle on the host, so the
    engine library is never mapped into its process."""
    import subprocess
    import sys
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'er16k', "
            "'--steps', '1', '--warmup', '0', '--ref-step-seconds', '0.1']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "print('ENGINE_MAPPED', 'libtc.so' in open('/proc/self/maps').read())")
    r = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ENGINE_MAPPED False" in r.stdout

"""Shared helpers for the reference-output fixtures
(tests/golden/reference_outputs.json, made by
tests/golden/make_reference_outputs.py from the reference's own graph.cc)."""
from __future__ import annotations

import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def _maker():
    spec = importlib.util.spec_from_file_location("make_reference_outputs", GOLDEN / "make_reference_outputs.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MAKER = _maker()


def fixtures() -> dict:
    return json.loads((GOLDEN / "reference_outputs.json").read_text())


def digest(a, dtype) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype).tobytes()).hexdigest()


def seeded_inputs():
    """name -> (rowptr, colidx, labels, classes, sort_neighbors), checked
    against the digests of the inputs the fixtures were made from."""
    rec = {r["name"]: r for r in fixtures()["seeded"]}
    out = {}
    for name, (rp, col, lab, classes, srt) in MAKER.seeded_graphs().items():
        assert digest(rp, np.int64) == rec[name]["input_rowptr_sha256"], name
        assert digest(col, np.int32) == rec[name]["input_colidx_sha256"], name
        out[name] = (rp, col, lab, classes, srt)
    return out


def golden_inputs(golden_cases):
    """(case name, rowptr, colidx, fixture record) for every golden case the
    reference accepted."""
    rec = {r["name"]: r for r in fixtures()["golden"]}
    out = []
    for c in golden_cases:
        r = rec[c["name"]]
        if "rejected_by_reference" in r:
            continue
        rp, col = MAKER.golden_csr(c)
        assert digest(rp, np.int64) == r["input_rowptr_sha256"], c["name"]
        assert digest(col, np.int32) == r["input_colidx_sha256"], c["name"]
        out.append((c["name"], rp, col, r))
    return out

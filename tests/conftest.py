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

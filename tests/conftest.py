import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def lib_built():
    """Build libwkgpu.so and the oracle in-tree (no-op when up to date)."""
    from wukonggpu_gb300 import build as wb
    import oracle
    wb.build()
    oracle.build(with_ref=True)
    return True


@pytest.fixture(scope="session")
def golden_small():
    return json.loads((GOLDEN / "small.json").read_text())


@pytest.fixture(scope="session")
def small_graph(lib_built):
    import wukonggpu_gb300 as W
    g = W.Graph(W.spec_small())
    s, p, o = g.arrays()
    return g, np.array(s), np.array(p), np.array(o)


@pytest.fixture(scope="session")
def small_oracle(small_graph):
    import oracle
    g, s, p, o = small_graph
    return oracle.Oracle(s, p, o, g.num_ids)


@pytest.fixture(scope="session")
def gpu_small(small_graph):
    """A device context holding the small graph's store (GPU tests only)."""
    import wukonggpu_gb300 as W
    g, s, p, o = small_graph
    rc = W.RCache(device=0)
    rc.build_store_graph(g)
    return rc

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "fdtd_golden.json").read_text())


@pytest.fixture(scope="session")
def golden_small():
    return dict(np.load(ROOT / "tests" / "golden" / "golden_small.npz"))


def params_of(case):
    """FDTD_PARAMS of a golden case as a ptask_gb300 FdtdParams."""
    from ptask_gb300._lib import FdtdParams
    p = FdtdParams()
    for f, _ in p._fields_:
        v = case["params"][f]
        setattr(p, f, v if isinstance(v, int) else float.fromhex(v))
    return p

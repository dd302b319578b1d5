import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libqg.so built for sm_103a")


@pytest.fixture(scope="session")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("CUDA GPU required for -m gpu tests")
    from query_on_opencl_fpga_gb300.api import Context

    c = Context()
    yield c
    c.close()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np

    d = ROOT / "tests" / "golden"
    meta = json.loads((d / "golden.json").read_text())
    arrs = dict(np.load(d / "golden.npz"))
    return meta, arrs

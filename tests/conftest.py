import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "reference_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ax():
    """The CUDA library, built in-tree if needed.  GPU tests fail (not skip)
    when the extension cannot be built or loaded."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arborx_gb300 import build as b

    b.build()
    import arborx_gb300

    arborx_gb300._lib.load()
    return arborx_gb300

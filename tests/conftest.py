import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build(ref=False)
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """Built product library on a CUDA device; GPU tests fail loudly without it."""
    import torch
    assert torch.cuda.is_available(), "GPU test collected on a machine without CUDA"
    from ohao_engine_gb300 import _build
    _build.build()
    import ohao_engine_gb300 as og
    og.load_library()
    return og

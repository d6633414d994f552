import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libgh1 kernels)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def cube_vol():
    import numpy as np
    d = np.load(os.path.join(ROOT, "tests", "golden", "cube_vol.npz"))
    return d["points"], d["tets"]


@pytest.fixture(scope="session")
def gpu():
    """Builds libgh1 (if needed) and returns the package; the CUDA path must load."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    from ngsolve_gb300 import build
    build.build()
    import ngsolve_gb300 as ng
    ng.context(0)
    return ng

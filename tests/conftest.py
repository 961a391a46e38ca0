import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def engine():
    """The built engine library (built in-tree on first use)."""
    from lj_gpu_gb300 import _build
    _build.build()
    import lj_gpu_gb300
    lj_gpu_gb300.lib()
    return lj_gpu_gb300


@pytest.fixture(scope="session")
def fixture_rho05():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "cpuref_rho0.5_L10.npz"))


@pytest.fixture(scope="session")
def fixture_rho1():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "cpuref_rho1_L8.npz"))

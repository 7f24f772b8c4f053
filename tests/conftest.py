import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    # Hermetic launch shapes: no tuning on first use (tests pin the shapes they
    # check; the tuner has its own tests) and a cache of the session's own.
    import tempfile
    os.environ.setdefault("MOSAIC_GB300_AUTOTUNE", "0")
    os.environ.setdefault("MOSAIC_GB300_CACHE", tempfile.mkdtemp(prefix="mosaic_gb300_tune_"))
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: full-size configuration (seconds to minutes)")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mosaic_gb300 import _lib
    _lib.load()          # builds if stale; raises if it cannot
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    return load

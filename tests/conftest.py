import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_small.npz")))


@pytest.fixture(scope="session")
def ctx():
    if not HAS_GPU:
        pytest.skip("no GPU")
    from __graft_entry__ import build
    build()
    import tapkee_gb300 as tk
    c = tk.Context(0)
    yield c
    c.close()

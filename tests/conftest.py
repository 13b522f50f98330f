import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libqbg.so")


def _ensure_built():
    """Build the oracle (and libqbg.so if absent) once per session."""
    from oracle import oracle as O
    if not os.path.exists(os.path.join(ROOT, "oracle", "libqbo.so")):
        O.build()
    if not os.path.exists(os.path.join(ROOT, "qball_gb300", "libqbg.so")):
        from qball_gb300 import build
        build.build()


_ensure_built()


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz"), allow_pickle=False))


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))

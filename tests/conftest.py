import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
# the reference's source tree, where present (CPU tests that read it skip
# without it; nothing that runs on a GPU reads it)
REF_TREE = os.environ.get("CFDWM_REFERENCE_TREE", "/root/reference")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def golden_cfg(g):
    """Parse the waveinput.dat text stored in a golden fixture with the oracle's parser."""
    from oracle import waveinput
    return waveinput.read_text(str(g["waveinput"]))


def norm_rel_err(a, b):
    """max|a-b| / max|b|: the normwise relative error used by every parity test."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    if den == 0.0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / den)


@pytest.fixture(scope="session")
def golden():
    return load_golden

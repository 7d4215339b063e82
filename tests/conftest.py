import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def rel_err(got, ref, floor=1e-2):
    """max |got-ref| / max(max|ref|, floor) over the whole array.  The floor
    keeps arrays that vanish by construction (the 0'-class F matrix on
    eigenstates) from turning rounding noise into a relative error."""
    got, ref = np.asarray(got), np.asarray(ref)
    scale = max(float(np.abs(ref).max()), floor)
    return float(np.abs(got - ref).max()) / scale


@pytest.fixture(scope="session")
def gpu_ctx():
    from nevpt2_gb300 import koopro
    return koopro.context()

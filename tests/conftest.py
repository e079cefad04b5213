import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libflame3d_gpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; skip when there is no GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from flame3d_mhd_gb300 import build
    build.build()
    from flame3d_mhd_gb300 import abi
    return abi.load()


def rel_linf(a, b, per_var=True, floor=0.0):
    """max |a-b| / max |b| per variable (first axis), with an optional absolute floor."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not per_var:
        return float(np.abs(a - b).max() / max(np.abs(b).max(), floor, 1e-300))
    out = 0.0
    for n in range(b.shape[0]):
        den = max(np.abs(b[n]).max(), floor, 1e-300)
        out = max(out, float(np.abs(a[n] - b[n]).max() / den))
    return out

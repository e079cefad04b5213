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


RHS_TOL = 1e-12  # the FP64 drop-in bar


def rhs_parity(P, Q, m, J, r):
    """Errors of an FP64 RHS r (interior cells compared) against the oracle: the FP64
    restatement and its extended-precision (long double) evaluation of the same formulas.

    flux-scaled: |a - b| / scale per variable, scale = max of J x the summed face fluxes the
    RHS differences (the size of the terms that cancel in it).
    """
    import numpy as np
    from oracle import oracle as orc
    I = (slice(None), slice(4, -4), slice(4, -4), slice(4, -4))
    ro = orc.rhs(P, Q, m, J)
    rl, scale = orc.rhs_ld(P, Q, m, J)

    def fs(a, b):
        return max(float(np.abs(a[n][I[1:]] - b[n][I[1:]]).max() / scale[n]) for n in range(5))
    return {"plain": rel_linf(r[I], ro[I]), "scaled": fs(r, ro), "scaled_ld": fs(r, rl), "orc_scaled_ld": fs(ro, rl),
            "gpu_ld": rel_linf(r[I], rl[I]), "orc_ld": rel_linf(ro[I], rl[I])}


def assert_rhs_parity(e, strict=False):
    """The FP64 RHS bar. Against the exact value of the reference's formulas (the oracle's
    extended-precision evaluation): flux-scaled error <= 1e-12, or, where the FP64 evaluation
    of those formulas cannot reach that (the FP64 oracle itself is further away: cancellation
    inside the formulas, e.g. the characteristic back-projection at rest), no more than 1.5x the
    FP64 oracle's own flux-scaled error. Against the FP64 oracle: plain relative L-inf <= 1e-12
    (strict) or <= 3x the oracle's own distance from the extended result."""
    msg = " ".join(f"{k} {v:.2e}" for k, v in e.items())
    assert e["scaled_ld"] <= max(RHS_TOL, 1.5 * e["orc_scaled_ld"]), msg
    assert e["gpu_ld"] <= max(RHS_TOL, 2.0 * e["orc_ld"]), msg
    assert e["plain"] <= max(RHS_TOL, 3.0 * e["orc_ld"]), msg
    if strict:
        assert e["plain"] <= RHS_TOL and e["scaled_ld"] <= RHS_TOL, msg

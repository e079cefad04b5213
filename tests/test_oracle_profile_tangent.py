"""The oracle's forward-mode derivative with respect to an inflow profile (dual numbers
seeded by orc_set_inflow_profile_tangent) against central differences of its own FP64 RHS
on a reduced compression ramp (component-wise reconstruction). The GPU adjoint's profile
cotangent is tested against this derivative (test_gpu_ramp_adjoint.py).

Tolerance: 1e-7 relative to the largest tangent component (h = 1e-6 relative to each
profile value: truncation ~h^2, rounding ~1e-16 / h)."""
import numpy as np
import pytest

from flame3d_mhd_gb300 import cases
from oracle import oracle as orc

NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


@pytest.fixture(scope="module")
def ramp():
    c = cases.compression_ramp(24, 16, 4, first_cell=1e-2, character=0)
    orc.set_inflow_profile(0, c["profile"])
    m, J, Q, U = orc.prepare(c["params"], c["Q"], c["x"], c["y"], c["z"])
    yield c, m, J, U
    orc.set_inflow_profile(0, None)
    orc.set_inflow_profile_tangent(0, None)


def _rhs_of_profile(c, m, J, U, prof):
    P = c["params"]
    orc.set_inflow_profile(0, prof)
    Q = orc.c2prim(P, U)
    Uf = U.copy()
    orc.fill_ghosts(P, Q, Uf)
    return orc.rhs(P, Q, m, J)


def test_profile_tangent_vs_central_difference(ramp):
    c, m, J, U = ramp
    P, prof = c["params"], c["profile"]
    rng = np.random.default_rng(5)
    d = rng.standard_normal(prof.shape) * np.abs(prof) * 1e-2
    orc.set_inflow_profile(0, prof)
    orc.set_inflow_profile_tangent(0, d)
    try:
        _, dr = orc.rhs_jvp_u(P, U, np.zeros_like(U), m, J)
    finally:
        orc.set_inflow_profile_tangent(0, None)
    h = 1e-4
    rp = _rhs_of_profile(c, m, J, U, prof + h * d)
    rm = _rhs_of_profile(c, m, J, U, prof - h * d)
    orc.set_inflow_profile(0, prof)
    fd = (rp - rm) / (2 * h)
    assert np.abs(dr[I]).max() > 0
    assert np.abs(fd[I] - dr[I]).max() <= 1e-7 * np.abs(dr[I]).max()

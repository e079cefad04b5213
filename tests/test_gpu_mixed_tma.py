"""The mixed form's TMA-staged sweeps against its direct-load sweeps.

Both compute the same arithmetic on the same FP32 inputs: the TMA sweeps only move the
stencil tiles (and, in the last sweep, the Phase C inputs: the two FP32 direction sums, J, U
and Un) into shared memory with cp.async.bulk.tensor and take their tiles from a counter.
So the RHS and the state after RK3 steps must be equal bit for bit. The direct-load sweeps are
selected by F3D_NO_TMA=1 when a context is created (and always for grids whose x extent with
ghosts is not a multiple of 4). Cases: the hybrid characteristic shock tube, a viscous
curvilinear state with the reference's boundary conditions, component-wise reconstruction,
and a ragged grid (no dimension a multiple of the tiles).
"""
import os

import numpy as np
import pytest
import torch

from flame3d_mhd_gb300.abi import PREC_MIXED
from flame3d_mhd_gb300.cases import params_copy
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from test_gpu_parity import dev, host, random_case, sod_case

pytestmark = pytest.mark.gpu

CASES = {
    "sod_char": lambda: sod_case((32, 16, 16)),
    "viscous_refbc_char": lambda: random_case(seed=51, bc="reference", viscous=1, rg=1.0, c_s=1e-2, t_s=1.0,
                                              phi1=0.02, phi2=0.1, phi3=0.4, spikes=10),
    "comp_hybrid": lambda: random_case(seed=52, character=0, phi1=0.02, phi2=0.1, phi3=0.4, spikes=20),
    "ragged_char": lambda: random_case(nx=36, ny=20, nz=44, seed=53, phi1=0.02, phi2=0.1, phi3=0.4, spikes=20),
}


def _mixed_run(c, no_tma: bool, steps: int = 3, dt: float = 1e-4):
    old = os.environ.get("F3D_NO_TMA")
    os.environ["F3D_NO_TMA"] = "1" if no_tma else "0"
    try:
        s = Flame3D(params_copy(c.P, precision=PREC_MIXED))
    finally:
        if old is None:
            del os.environ["F3D_NO_TMA"]
        else:
            os.environ["F3D_NO_TMA"] = old
    s.set_metrics(c.md, c.Jd)
    r = host(s.rhs(dev(c.Q)))
    U, Un, Q = dev(c.U), torch.zeros_like(dev(c.U)), dev(c.Q)
    with side_stream() as stream:
        s.time_step(U, Un, Q, dt, steps)
    stream.synchronize()
    assert s.check_finite(U)  # also reports a sweep whose tile copies did not complete
    out = host(U), host(Q)
    s.close()
    return r, out


@pytest.mark.parametrize("name", sorted(CASES))
def test_tma_sweeps_equal_direct_loads(gpu_lib, name):
    c = CASES[name]()
    r_tma, (U_tma, Q_tma) = _mixed_run(c, no_tma=False)
    r_dir, (U_dir, Q_dir) = _mixed_run(c, no_tma=True)
    assert np.isfinite(r_tma).all()
    assert np.array_equal(r_tma, r_dir)
    assert np.array_equal(U_tma, U_dir)
    assert np.array_equal(Q_tma, Q_dir)
    c.close()

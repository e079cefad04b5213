"""The two oracle-checkable configurations at their full sizes and step counts, GPU against
the oracle from the same initial state:

- Taylor-Green vortex, inviscid, uniform periodic 64^3 on [0, 2pi)^3, Mach 0.1, WENO5
  everywhere, Steger-Warming, SSP-RK3 at CFL 0.5 for 100 steps: the RHS of the initial
  state and the state after 100 steps; plus conservation of mass, momentum and energy over
  the run (periodic faces telescope);
- shock tube on the perturbed curvilinear grid, 256x64x64, hybrid WENO7/WENO5/UP7 with the
  sensor active, characteristic, inviscid, 200 steps: the state after 200 steps.

Tolerances, written per check:
- RHS: conftest.assert_rhs_parity, as test_gpu_parity (against the oracle's extended-
  precision evaluation relative to the flux scale <= 1e-12, or <= 1.5x the FP64 oracle's own
  error where the FP64 evaluation of the formulas cannot reach 1e-12; against the FP64 oracle
  within 3x its own rounding);
- states after N steps: L-inf of the difference relative to the largest state component,
  <= 1e-11 for the vortex and <= 1e-10 for the shock tube. Both sides round differently
  (FMA contraction, WENO weight normalisation) by ~1e-16 relative per operation; the
  bounds allow that to accumulate over 300 / 600 RHS evaluations with the growth a
  shock-capturing scheme gives it near the discontinuities;
- conservation: each integral's change over the run relative to the integral's scale,
  <= 1e-12.
"""
import numpy as np
import pytest
import torch

from conftest import assert_rhs_parity, rel_linf, rhs_parity
from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def _run_gpu(P, m, J, Q, U, dt, steps):
    s = Flame3D(P)
    s.set_metrics([dev(a) for a in m], dev(J))
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream() as stream:
        s.time_step(Ud, Und, Qd, dt, steps)
    stream.synchronize()
    r = host(s.rhs(dev(Q)))
    out = host(Ud)
    s.close()
    return out, r


def _integrals(U, J):
    w = 1.0 / J[I[1:]]
    return np.array([float((U[n][I[1:]] * w).sum()) for n in range(5)])


def test_tgv64_rhs_and_100_steps(gpu_lib):
    c = cases.tgv(64)
    P = c["params"]
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    dt, steps = c["dt"], 100
    Ug, rg = _run_gpu(P, m, J, Q, U, dt, steps)
    # RHS of the initial state
    assert_rhs_parity(rhs_parity(P, Q, m, J, rg))
    # state after 100 steps
    Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
    orc.rk3(P, steps, dt, Uo, Uno, Qo, m, J)
    assert rel_linf(Ug[I], Uo[I], per_var=False) <= 1e-11
    # conservation over the run: mass and energy against their own integrals, momentum
    # against the momentum scale (its integrals are zero)
    i0, i1 = _integrals(U, J), _integrals(Ug, J)
    vol = float((1.0 / J[I[1:]]).sum())
    mom_scale = float(np.abs(U[1:4][I]).max()) * vol
    for n in (0, 4):
        assert abs(i1[n] - i0[n]) <= 1e-12 * abs(i0[n]), (n, i0[n], i1[n])
    for n in (1, 2, 3):
        assert abs(i1[n] - i0[n]) <= 1e-12 * mom_scale, (n, i0[n], i1[n])


def test_sod_curvilinear_256x64x64_200_steps(gpu_lib):
    c = cases.sod(256, 64, 64)
    P = c["params"]
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    dt, steps = c["dt"], 200
    Ug, rg = _run_gpu(P, m, J, Q, U, dt, steps)
    # RHS of the initial state
    assert_rhs_parity(rhs_parity(P, Q, m, J, rg))
    Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
    orc.rk3(P, steps, dt, Uo, Uno, Qo, m, J)
    assert np.isfinite(Ug).all()
    err = rel_linf(Ug[I], Uo[I], per_var=False)
    assert err <= 1e-10, err

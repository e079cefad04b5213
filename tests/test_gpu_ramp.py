"""Compression ramp (viscous Mach 2.9, 24-degree ramp, isothermal wall, per-point inflow
profile) on a reduced grid: the inflow-profile ghost rule bitwise against the oracle, FP64
RK3 steps against the oracle, and mixed precision against FP64 by wall pressure and skin
friction.

Tolerances, written per check:
- ghost fill: bitwise (integer-exact rule chain; the same IEEE operations on both sides);
- FP64 state after 50 steps: L-inf relative to the largest state component <= 1e-11 (both
  sides round differently by ~1e-16 per operation over 150 RHS evaluations);
- mixed vs FP64 after 100 steps: wall pressure within 1e-5 relative (max over the wall
  against the largest wall pressure, and the wall mean); skin friction within 1e-4
  relative to its largest magnitude (it differences velocities across the first cell,
  where FP32 fluxes leave their last-bit errors).
"""
import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import F3D_ERR_ARG, F3D_ERR_STATE, PREC_MIXED, F3DError
from flame3d_mhd_gb300.cases import params_copy
from flame3d_mhd_gb300.ramp import skin_friction, wall_pressure
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def ramp():
    c = cases.compression_ramp(64, 32, 8, first_cell=1e-2)
    orc.set_inflow_profile(0, c["profile"])
    m, J, Q, U = orc.prepare(c["params"], c["Q"], c["x"], c["y"], c["z"])
    yield c, m, J, Q, U
    orc.set_inflow_profile(0, None)


def _solver(c, m, J, precision=0):
    s = Flame3D(params_copy(c["params"], precision=precision))
    s.set_metrics([dev(a) for a in m], dev(J))
    prof = dev(c["profile"])
    s.set_inflow_profile(0, prof)
    return s


def test_inflow_profile_fill_bitwise(gpu_lib, ramp):
    c, m, J, Q, U = ramp
    s = _solver(c, m, J)
    rng = np.random.default_rng(5)
    g = np.ones(Q.shape[1:], bool)
    g[NG:-NG, NG:-NG, NG:-NG] = False
    Qi, Ui = Q.copy(), U.copy()
    Qi[:, g] = rng.uniform(-5, 5, (6, g.sum()))
    Ui[:, g] = rng.uniform(-5, 5, (5, g.sum()))
    Qd, Ud = dev(Qi), dev(Ui)
    s.fillGhost(Qd, Ud)
    Qo, Uo = Qi.copy(), Ui.copy()
    orc.fill_ghosts(c["params"], Qo, Uo)
    assert np.array_equal(host(Qd), Qo)
    assert np.array_equal(host(Ud), Uo)
    s.close()


def test_ramp_fp64_steps_vs_oracle(gpu_lib, ramp):
    c, m, J, Q, U = ramp
    s = _solver(c, m, J)
    r = host(s.rhs(dev(Q)))
    ro = orc.rhs(c["params"], Q, m, J)
    rl, _ = orc.rhs_ld(c["params"], Q, m, J)
    orc_ld = rel_linf(ro[I], rl[I])
    assert rel_linf(r[I], ro[I]) <= max(1e-12, 3.0 * orc_ld)
    assert rel_linf(r[I], rl[I]) <= max(1e-12, 2.0 * orc_ld)
    steps, dt = 50, c["dt"]
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream() as stream:
        s.time_step(Ud, Und, Qd, dt, steps)
    stream.synchronize()
    Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
    orc.rk3(c["params"], steps, dt, Uo, Uno, Qo, m, J)
    assert rel_linf(host(Ud)[I], Uo[I], per_var=False) <= 1e-11
    s.close()


def _advance(c, m, J, Q, U, precision, steps):
    s = _solver(c, m, J, precision)
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream() as stream:
        s.time_step(Ud, Und, Qd, c["dt"], steps)
    stream.synchronize()
    assert s.check_finite(Ud)
    out = host(Qd)
    s.close()
    return out


def test_ramp_mixed_wall_pressure_and_skin_friction(gpu_lib, ramp):
    c, m, J, Q, U = ramp
    Q64 = _advance(c, m, J, Q, U, 0, 100)
    Q32 = _advance(c, m, J, Q, U, PREC_MIXED, 100)
    pw64, pw32 = wall_pressure(Q64), wall_pressure(Q32)
    assert pw64.max() > 1.2 * c["wall"]["p_inf"]  # the ramp compression is there
    assert float(np.abs(pw32 - pw64).max() / np.abs(pw64).max()) <= 1e-5
    assert abs(pw32.mean() - pw64.mean()) <= 1e-5 * abs(pw64.mean())
    cf64 = skin_friction(Q64, c["x"], c["y"], c["wall"])
    cf32 = skin_friction(Q32, c["x"], c["y"], c["wall"])
    assert float(np.abs(cf32 - cf64).max() / np.abs(cf64).max()) <= 1e-4


def test_inflow_profile_errors(gpu_lib, ramp):
    c, m, J, Q, U = ramp
    s = Flame3D(c["params"])
    s.set_metrics([dev(a) for a in m], dev(J))
    with pytest.raises(F3DError) as e:
        s.rhs(dev(Q))  # profile face without its profile
    assert e.value.code == F3D_ERR_STATE
    with pytest.raises(F3DError) as e:  # face 1 (x+) is zero-gradient
        s._check(s.lib.f3d_set_inflow_profile(s._h, 1, None, None))
    assert e.value.code == F3D_ERR_ARG
    s.close()

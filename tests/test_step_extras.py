"""Local time stepping, explicit filters and LES (utils.jl:73-315, div.jl:52-101,
viscous.jl:66-106): known answers of the oracle on the CPU, then the GPU against the oracle.

Tolerances: known answers to rounding (1e-14 of the field); GPU local dt and one filter pass
within 1e-13 relative (the same formulas, FMA contraction); RHS with LES and states after
steps with local time stepping or filtering within 1e-12 relative, as the other parity tests."""
import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300.abi import (BC_PERIODIC, F3D_ERR_UNSUPPORTED, FILTER_LINEAR, FILTER_NONLINEAR,
                                   LES_SMAGORINSKY, LES_WALE, F3DError, make_params)
from oracle import oracle as orc

NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
PER = [dict(kind=BC_PERIODIC)] * 6


def _case(seed=3, n=(18, 14, 12), spikes=0, **kw):
    from test_gpu_parity import curvilinear_coords, random_state
    P = make_params(*n, bc=PER, character=0, **kw)
    x, y, z = curvilinear_coords(P)
    m, J, Q, U = orc.prepare(P, random_state(P, seed, spikes), x, y, z)
    return P, m, J, Q, U


# ---- CPU: known answers ------------------------------------------------------------------
def test_linear_filter_keeps_constants_and_removes_the_grid_mode():
    P = make_params(12, 12, 12, bc=PER, filter=FILTER_LINEAR)
    shape = (5, P.nz + 8, P.ny + 8, P.nx + 8)
    U = np.ones(shape) * np.array([1.0, 0.2, -0.1, 0.3, 2.5])[:, None, None, None]
    Q = np.zeros((6, *shape[1:]))
    Uf, Un = U.copy(), np.zeros_like(U)
    orc.filter_pass(P, Uf, Un, Q)
    assert np.abs(Uf - U).max() <= 1e-14
    # (-1)^i on top of a constant: the 8th-order filter's response at pi is exactly 1, so
    # with s0 = 1 the x pass removes the mode from the interior. The y and z passes then see
    # constants except within 4 cells of the y / z boundaries, where their stencils reach
    # ghost cells that no pass refills (as in the reference): check the core
    k, j, i = np.meshgrid(*[np.arange(s) for s in shape[1:]], indexing="ij")
    mode = (-1.0) ** i
    Um = U + 0.01 * mode
    orc.filter_pass(P, Um, Un, Q)
    core = (slice(None), slice(2 * NG, -2 * NG), slice(2 * NG, -2 * NG), slice(NG, -NG))
    assert np.abs(Um[core] - U[core]).max() <= 1e-14


def test_shock_filter_leaves_smooth_pressure_alone():
    P, m, J, Q, U = _case(filter=FILTER_NONLINEAR)
    Q = Q.copy()
    Q[4] = 0.7  # uniform pressure: the sensor is 0 everywhere
    Uf, Un = U.copy(), np.zeros_like(U)
    orc.filter_pass(P, Uf, Un, Q)
    assert np.array_equal(Uf, U)


def test_local_dt_formula():
    P, m, J, Q, U = _case(lts=1, lts_cfl=0.4)
    dt = orc.local_dt(P, Q, m, J)
    c = np.sqrt(P.gamma * P.rg * Q[5])
    S = [np.sqrt(m[3 * d] ** 2 + m[3 * d + 1] ** 2 + m[3 * d + 2] ** 2) for d in range(3)]
    ref = 0.4 * np.minimum(np.minimum(1 / J / S[0] / (Q[1] + c), 1 / J / S[1] / (Q[2] + c)), 1 / J / S[2] / (Q[3] + c))
    assert np.abs(dt[I[1:]] - ref[I[1:]]).max() <= 1e-14 * np.abs(ref[I[1:]]).max()


# ---- GPU against the oracle ---------------------------------------------------------------
def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def _solver(P, m, J):
    from flame3d_mhd_gb300.solver import Flame3D
    s = Flame3D(P)
    s.set_metrics([dev(a) for a in m], dev(J))
    return s


@pytest.mark.gpu
def test_gpu_local_dt(gpu_lib):
    P, m, J, Q, U = _case(lts=1, lts_cfl=0.4)
    s = _solver(P, m, J)
    dt = host(s.compute_dt(dev(Q)))
    ref = orc.local_dt(P, Q, m, J)
    assert rel_linf(dt[I[1:]][None], ref[I[1:]][None]) <= 1e-13
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [FILTER_LINEAR, FILTER_NONLINEAR])
def test_gpu_filter_pass(gpu_lib, mode):
    P, m, J, Q, U = _case(spikes=15, filter=mode, filter_rth=1e-4)
    s = _solver(P, m, J)
    Ud, Und = dev(U), dev(np.zeros_like(U))
    s.filter(Ud, Und, dev(Q))
    Uo, Uno = U.copy(), np.zeros_like(U)
    orc.filter_pass(P, Uo, Uno, Q)
    assert rel_linf(host(Ud)[I], Uo[I]) <= 1e-13
    assert not np.array_equal(Uo[I], U[I])  # the filter acted
    s.close()


def _steps(P, m, J, Q, U, dt, steps):
    from flame3d_mhd_gb300.solver import side_stream
    s = _solver(P, m, J)
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream():
        s.time_step(Ud, Und, Qd, dt, steps)
    torch.cuda.synchronize()
    out = host(Ud)
    s.close()
    Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
    orc.rk3(P, steps, dt, Uo, Uno, Qo, m, J)
    return out, Uo


@pytest.mark.gpu
def test_gpu_lts_steps(gpu_lib):
    P, m, J, Q, U = _case(lts=1, lts_cfl=0.3, viscous=0)
    Ug, Uo = _steps(P, m, J, Q, U, 0.0, 3)
    assert not np.array_equal(Uo[I], U[I])
    assert rel_linf(Ug[I], Uo[I], per_var=False) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [FILTER_LINEAR, FILTER_NONLINEAR])
def test_gpu_filtered_steps(gpu_lib, mode):
    P, m, J, Q, U = _case(spikes=10, viscous=0, filter=mode, filter_interval=2, filter_rth=1e-4)
    Ug, Uo = _steps(P, m, J, Q, U, 1e-3, 4)
    assert rel_linf(Ug[I], Uo[I], per_var=False) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("les", [LES_SMAGORINSKY, LES_WALE])
def test_gpu_les_rhs(gpu_lib, les):
    P, m, J, Q, U = _case(seed=7, viscous=1, les=les, rg=1.0, c_s=1e-2, t_s=1.0)
    s = _solver(P, m, J)
    r = host(s.rhs(dev(Q)))
    ro = orc.rhs(P, Q, m, J)
    rl, _ = orc.rhs_ld(P, Q, m, J)
    orc_ld = rel_linf(ro[I], rl[I])
    assert rel_linf(r[I], ro[I]) <= max(1e-12, 3.0 * orc_ld)
    # the eddy viscosity changes the answer
    from flame3d_mhd_gb300.cases import params_copy
    assert rel_linf(orc.rhs(params_copy(P, les=0), Q, m, J)[I], ro[I]) > 1e-6
    with pytest.raises(F3DError) as e:
        s.rhs_vjp(dev(U), dev(np.zeros_like(U)))
    assert e.value.code == F3D_ERR_UNSUPPORTED
    s.close()

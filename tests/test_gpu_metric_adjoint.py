"""Metric and Jacobian cotangents of the discrete adjoint (f3d_set_metrics_cotangent):
dot products <metrics_bar, dm> + <J_bar, dJ> = <L_bar, dL/d(metrics, J) . (dm, dJ)> against
the oracle's forward-mode dual numbers seeded with metric tangents, for one RHS (inviscid
hybrid with SW and LF splitting, WENO5 everywhere, viscous with Dirichlet, adiabatic-wall and
isothermal-wall faces) and for two chained RK3 steps.

Tolerance: 1e-10 relative to the sum of |terms| (both sides exact derivatives of the same
branch-frozen FP64 scheme; the GPU adds its contributions with FP64 atomics).

The cases have no zero-gradient faces: their ghost cells repeat the last interior state, so
a WENO stencil in the ghost layers sees split fluxes that differ only through the ghost
metrics, its smoothness indicators sit near the eps floor and the derivative with respect to
those metrics is set by rounding (double and long-double central differences of the same
RHS disagree by 2% there, and so do the dual numbers); with UP7 faces there, or Dirichlet
faces, all three agree to 1e-9."""
import numpy as np
import pytest

from flame3d_mhd_gb300.abi import BC_DIRICHLET, BC_PERIODIC, BC_WALL_ADIABATIC, BC_WALL_ISOTHERMAL, make_params
from flame3d_mhd_gb300.solver import Flame3D
from oracle import oracle as orc
from test_gpu_adjoint import CASES as STATE_CASES
from test_gpu_adjoint import _interior_random
from test_gpu_parity import curvilinear_coords, dev, host, random_state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


FS = dict(kind=BC_DIRICHLET, rho=1.0, u=0.5, v=0.0, w=0.0, p=1.0 / 1.4)
PER = dict(kind=BC_PERIODIC)


def _walls(seed, wall):
    P = make_params(20, 14, 12, character=0, viscous=1, rg=1.0, c_s=1e-2, t_s=1.0, bc=[FS, FS, wall, FS, PER, PER])
    x, y, z = curvilinear_coords(P)
    Q0 = random_state(P, seed, 0)
    with np.errstate(invalid="ignore", divide="ignore"):  # ghost cells hold zeros until the fill
        Q0[5] = Q0[4] / (Q0[0] * P.rg)
    return P, Q0, x, y, z


CASES = {k: STATE_CASES[k] for k in ("tgv16_weno5", "curvi_hybrid_sw", "curvi_hybrid_lf", "curvi_char_hybrid_sw",
                                     "curvi_char_vl", "curvi_comp_ausm")}
CASES["curvi_dirichlet_adiabatic_viscous"] = lambda: _walls(35, dict(kind=BC_WALL_ADIABATIC))
CASES["curvi_dirichlet_isothermal_viscous"] = lambda: _walls(36, dict(kind=BC_WALL_ISOTHERMAL, t_wall=1.0))


def _setup(name):
    P, Q0, x, y, z = CASES[name]()
    m, J, Q, U = orc.prepare(P, Q0, x, y, z)
    s = Flame3D(P)
    keep = ([dev(a) for a in m], dev(J))
    s.set_metrics(*keep)
    return P, m, J, Q, U, s, keep


def _tangents(m, J, seed):
    rng = np.random.default_rng(seed)
    dm = [rng.standard_normal(a.shape) * np.abs(a).max() * 1e-3 for a in m]
    dJ = rng.standard_normal(J.shape) * np.abs(J).max() * 1e-3
    return dm, dJ


def _bars(s):
    mb = [s.field(1) for _ in range(9)]
    Jb = s.field(1)
    s.set_metrics_cotangent(mb, Jb)
    return mb, Jb


def _lhs(mb, Jb, dm, dJ):
    terms = [host(a) * b for a, b in zip(mb, dm)] + [host(Jb) * dJ]
    return float(sum(t.sum() for t in terms)), float(sum(np.abs(t).sum() for t in terms))


@pytest.mark.parametrize("name", sorted(CASES))
def test_rhs_metric_cotangent_dot_product(gpu_lib, name):
    P, m, J, Q, U, s, keep = _setup(name)
    dm, dJ = _tangents(m, J, 5)
    Lb = _interior_random(U.shape, 6)
    _, jvp = orc.rhs_jvp_m(P, Q, m, dm, J, dJ)
    mb, Jb = _bars(s)
    s.rhs_vjp(dev(U), dev(Lb))
    s.set_metrics_cotangent(None)
    lhs, scale_l = _lhs(mb, Jb, dm, dJ)
    rhs = float((Lb[I] * jvp[I]).sum())
    scale = max(scale_l, float(np.abs(Lb[I] * jvp[I]).sum()))
    assert rhs != 0.0
    assert abs(lhs - rhs) <= 1e-10 * scale, (lhs, rhs)
    s.close()


@pytest.mark.parametrize("name", ["tgv16_weno5", "curvi_hybrid_sw", "curvi_dirichlet_isothermal_viscous"])
def test_rk3_steps_metric_cotangent_dot_product(gpu_lib, name):
    P, m, J, Q, U, s, keep = _setup(name)
    dt = 1e-3 if name.startswith("tgv") else 2e-4
    steps = 2
    dm, dJ = _tangents(m, J, 7)
    Ub = _interior_random(U.shape, 8)
    _, jvp = orc.rk3_jvp_m(P, steps, dt, U, m, dm, J, dJ)
    states = [dev(U)]
    Un, Qd = s.field(5), s.field(6)
    for _ in range(steps - 1):
        Ut = states[-1].clone()
        s.q_from_u(Ut, Qd)
        s.time_step(Ut, Un, Qd, dt, 1)
        states.append(Ut)
    mb, Jb = _bars(s)
    g = dev(Ub)
    for Ut in reversed(states):
        g = s.rk3_step_vjp(dt, Ut, g)
    s.set_metrics_cotangent(None)
    lhs, scale_l = _lhs(mb, Jb, dm, dJ)
    rhs = float((Ub[I] * jvp[I]).sum())
    scale = max(scale_l, float(np.abs(Ub[I] * jvp[I]).sum()))
    assert rhs != 0.0
    assert abs(lhs - rhs) <= 1e-10 * scale, (lhs, rhs)
    s.close()

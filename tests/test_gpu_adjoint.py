"""Discrete adjoint: hand-written VJP kernels against the oracle's forward-mode dual numbers
(dot-product test) and against central finite differences through checkpointed RK3
trajectories.

Tolerances: dot products agree to 1e-10 relative (both sides are exact derivatives of the
same branch-frozen FP64 scheme, so only rounding separates them); finite differences
with h = 1e-6 agree to 1e-6 relative (their own truncation and cancellation error).
"""
import numpy as np
import pytest
import torch

from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import BC_PERIODIC, make_params
from flame3d_mhd_gb300.adjoint import RK3Rollout, gradient
from flame3d_mhd_gb300.solver import Flame3D
from oracle import oracle as orc
from test_gpu_parity import curvilinear_coords, dev, host, random_state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def _random(seed, spikes=0, bc="periodic", n=(20, 14, 12), **kw):
    if bc == "periodic":
        kw["bc"] = [dict(kind=BC_PERIODIC)] * 6
    kw.setdefault("character", 0)
    P = make_params(*n, **kw)
    x, y, z = curvilinear_coords(P)
    return P, random_state(P, seed, spikes), x, y, z


def _random_transonic(seed, **kw):
    """A random curvilinear state streaming along x at Mach 0.6 .. 1.6, so the Mach-number
    splits take both their subsonic and their supersonic branches."""
    P, Q0, x, y, z = _random(seed, **kw)
    rng = np.random.default_rng(seed + 100)
    c = np.sqrt(1.4 * np.maximum(Q0[4], 1e-12) / np.maximum(Q0[0], 1e-12))
    Q0[1] += c * rng.uniform(0.6, 1.6, Q0[1].shape) * (Q0[0] > 0)
    return P, Q0, x, y, z


CASES = {
    "tgv16_weno5": lambda: (lambda c: (c["params"], c["Q"], c["x"], c["y"], c["z"]))(cases.tgv(16, character=0)),
    "curvi_hybrid_sw": lambda: _random(31, spikes=20, phi1=0.02, phi2=0.1, phi3=0.4, viscous=0),
    "curvi_hybrid_lf": lambda: _random(32, spikes=20, phi1=0.02, phi2=0.1, phi3=0.4, viscous=0, split="LF"),
    "curvi_refbc_viscous": lambda: _random(33, bc="reference", viscous=1, rg=1.0, c_s=1e-2, t_s=1.0),
    "curvi_isothermal_viscous": lambda: _random(
        34, viscous=1, rg=1.0, c_s=1e-2, t_s=1.0,
        bc=[dict(kind=2), dict(kind=2), dict(kind=4, t_wall=0.8), dict(kind=1, rho=1.0, u=0.2, v=0.0, w=0.0, p=0.7),
            dict(kind=0), dict(kind=0)]),
    # characteristic-wise reconstruction (the reference's default, run.jl:68) with all four
    # branches, and the van Leer and AUSM splits in both reconstruction modes
    "curvi_char_hybrid_sw": lambda: _random(37, spikes=20, phi1=0.02, phi2=0.1, phi3=0.4, character=1),
    "curvi_char_hybrid_lf": lambda: _random(38, spikes=20, phi1=0.02, phi2=0.1, phi3=0.4, character=1, split="LF"),
    "curvi_char_vl": lambda: _random(39, spikes=10, phi1=0.02, phi2=0.1, phi3=0.4, character=1, split="VL"),
    "curvi_char_ausm": lambda: _random(40, spikes=10, phi1=0.02, phi2=0.1, phi3=0.4, character=1, split="AUSM"),
    "curvi_comp_vl": lambda: _random(41, spikes=10, phi1=0.02, phi2=0.1, phi3=0.4, split="VL"),
    "curvi_comp_ausm": lambda: _random(42, spikes=10, phi1=0.02, phi2=0.1, phi3=0.4, split="AUSM"),
    "curvi_char_vl_transonic": lambda: _random_transonic(44, phi1=0.02, phi2=0.1, phi3=0.4, character=1, split="VL"),
    "curvi_comp_ausm_transonic": lambda: _random_transonic(45, phi1=0.02, phi2=0.1, phi3=0.4, split="AUSM"),
    "curvi_char_refbc_viscous": lambda: _random(43, bc="reference", viscous=1, rg=1.0, c_s=1e-2, t_s=1.0,
                                                character=1, phi1=0.0, phi2=0.05, phi3=np.inf),
}


def _interior_random(shape, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(shape)
    a[I] = rng.standard_normal(a[I].shape)
    return a


def _setup(name):
    P, Q0, x, y, z = CASES[name]()
    m, J, Q, U = orc.prepare(P, Q0, x, y, z)
    s = Flame3D(P)
    md, Jd = [dev(a) for a in m], dev(J)
    s.set_metrics(md, Jd)
    return P, m, J, Q, U, s, (md, Jd)


@pytest.mark.parametrize("name", sorted(CASES))
def test_rhs_vjp_dot_product_vs_dual_jvp(gpu_lib, name):
    P, m, J, Q, U, s, keep = _setup(name)
    dU = _interior_random(U.shape, 1) * 1e-3 * np.abs(U[I]).max()
    Lb = _interior_random(U.shape, 2)
    _, jvp = orc.rhs_jvp_u(P, U, dU, m, J)
    vjp = host(s.rhs_vjp(dev(U), dev(Lb)))
    lhs = float((vjp[I] * dU[I]).sum())
    rhs = float((Lb[I] * jvp[I]).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(Lb[I] * jvp[I]).sum(), (lhs, rhs)
    s.close()


@pytest.mark.parametrize("name", ["tgv16_weno5", "curvi_hybrid_sw", "curvi_refbc_viscous", "curvi_char_hybrid_sw",
                                  "curvi_char_vl"])
def test_rk3_step_vjp_dot_product(gpu_lib, name):
    P, m, J, Q, U, s, keep = _setup(name)
    dt = 1e-3 if name.startswith("tgv") else 2e-4
    steps = 2
    dU = _interior_random(U.shape, 3) * 1e-3 * np.abs(U[I]).max()
    Ub = _interior_random(U.shape, 4)
    _, jvp = orc.rk3_jvp_u(P, steps, dt, U, dU, m, J)
    # chain the step VJPs through the recomputed trajectory
    states = [dev(U)]
    Un, Qd = s.field(5), s.field(6)
    for _ in range(steps - 1):
        Ut = states[-1].clone()
        s.q_from_u(Ut, Qd)
        s.time_step(Ut, Un, Qd, dt, 1)
        states.append(Ut)
    g = dev(Ub)
    for Ut in reversed(states):
        g = s.rk3_step_vjp(dt, Ut, g)
    vjp = host(g)
    lhs = float((vjp[I] * dU[I]).sum())
    rhs = float((Ub[I] * jvp[I]).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(Ub[I] * jvp[I]).sum(), (lhs, rhs)
    s.close()


def _kinetic(Ut, J):
    rho = Ut[0][I[1:]]
    return float(((0.5 * (Ut[1][I[1:]] ** 2 + Ut[2][I[1:]] ** 2 + Ut[3][I[1:]] ** 2) / rho) / J[I[1:]]).sum())


def _kinetic_grad(Ut, Jd):
    """d/dU of sum over interior cells of (|rho u|^2 / (2 rho)) / J."""
    g = torch.zeros_like(Ut)
    r = Ut[0][I[1:]]
    m2 = Ut[1][I[1:]] ** 2 + Ut[2][I[1:]] ** 2 + Ut[3][I[1:]] ** 2
    w = 1.0 / Jd[I[1:]]
    g[0][I[1:]] = -0.5 * m2 / r ** 2 * w
    for k in (1, 2, 3):
        g[k][I[1:]] = Ut[k][I[1:]] / r * w
    return g


def smooth_generic_state(n=12):
    """Taylor-Green vortex plus smooth 3-D variations of rho, w and p and a drift. The plain
    vortex has flux components that are exactly constant along z (where cos 2x + cos 2y = 0),
    whose WENO smoothness indicators are exactly 0; there the weights sit at eps = 1e-16 and
    vary at a scale no finite difference resolves, although the exact derivative (linear
    weights) is well defined. The drift keeps contravariant velocities off the kink of the
    Steger-Warming split at zero."""
    c = cases.tgv(n, character=0)
    P = c["params"]
    X, Y, Z = c["x"], c["y"], c["z"]
    Q0 = c["Q"].copy()
    Q0[0][I[1:]] = (1 + 0.05 * np.sin(X + 2 * Y + 3 * Z))[I[1:]]
    Q0[1][I[1:]] += 0.03
    Q0[2][I[1:]] += 0.02
    Q0[3][I[1:]] += (0.05 + 0.02 * np.cos(2 * X - Y + Z))[I[1:]]
    Q0[4][I[1:]] *= (1 + 0.03 * np.cos(3 * X + Y - 2 * Z))[I[1:]]
    Q0[5][I[1:]] = Q0[4][I[1:]] / (Q0[0][I[1:]] * P.rg)
    return P, Q0, X, Y, Z, c["dt"]


def test_kinetic_energy_gradient_vs_central_differences(gpu_lib):
    """J = volume-integrated kinetic energy after 9 RK3 steps (WENO5 component-wise), gradient
    by sqrt(N)-checkpointed step VJPs (checkpoints every 3 steps), checked along 8 seeded
    Gaussian directions, entries scaled per variable by max |U| (not normalised, as the adjoint
    configuration states them): against the exact directional derivative of the oracle's
    forward-mode dual numbers through the 9 steps (1e-10), and against central differences with
    h = 1e-8 (1e-6). On this 12^3 grid a step of h = 1e-6 along such a direction is far enough
    from linear that the differences' own truncation error is 2e-5 .. 4.5e-4 (falling as h^2:
    8e-8 at h = 1e-8)."""
    P, Q0, X, Y, Z, dt = smooth_generic_state(12)
    m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
    s = Flame3D(P)
    md, Jd = [dev(a) for a in m], dev(J)
    s.set_metrics(md, Jd)
    nsteps = 9
    U0 = dev(U)
    UN, grad = gradient(s, U0, dt, nsteps, lambda UN: _kinetic_grad(UN, Jd), every=3)

    def J_of(Ustart):
        Ut = Ustart.clone()
        Un, Qd = s.field(5), s.field(6)
        s.q_from_u(Ut, Qd)
        s.time_step(Ut, Un, Qd, dt, nsteps)
        return _kinetic(host(Ut), J)

    h = 1e-8
    rng = np.random.default_rng(2024)
    for k in range(8):
        d = np.zeros(U.shape)
        d[I] = rng.standard_normal(d[I].shape) * np.abs(U[I]).max(axis=(1, 2, 3), keepdims=True)
        dd = dev(d)
        ad = float((grad * dd).sum())
        UN_o, dUN = orc.rk3_jvp_u(P, nsteps, dt, U, d, m, J)
        jv = float((host(_kinetic_grad(dev(UN_o), Jd))[I] * dUN[I]).sum())
        assert abs(jv - ad) <= 1e-10 * abs(ad), (k, jv, ad)
        fd = (J_of(U0 + h * dd) - J_of(U0 - h * dd)) / (2 * h)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    s.close()


def test_rk3_rollout_autograd(gpu_lib):
    """The torch.autograd wrapper returns the same gradient as the explicit driver."""
    c = cases.tgv(8, character=0)
    P = c["params"]
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    s = Flame3D(P)
    md, Jd = [dev(a) for a in m], dev(J)
    s.set_metrics(md, Jd)
    U0 = dev(U).requires_grad_(True)
    UN = RK3Rollout.apply(U0, s, c["dt"], 5, 2)
    w = dev(_interior_random(U.shape, 9))
    (UN * w).sum().backward()
    _, g2 = gradient(s, dev(U), c["dt"], 5, lambda _: w, every=2)
    assert torch.allclose(U0.grad, g2, rtol=1e-12, atol=1e-14 * float(g2.abs().max()))
    s.close()


def test_vjp_dot_products_at_full_size(gpu_lib):
    """The adjoint configuration's own grid and physics: viscous curvilinear Taylor-Green
    vortex 128^3 (amplitude 0.05, Re 1600, Mach 0.1), FP64, component-wise hybrid, with the
    smooth 3-D variations and drift of smooth_generic_state. Dot products of the RHS VJP and
    of one RK3 step VJP against the oracle's forward-mode dual numbers, 1e-10 (measured
    3e-19). Without the drift the vortex's symmetry puts contravariant velocities exactly on
    the Steger-Warming kink (E = +-0) at some cells, where the two exact derivatives take
    different one-sided values (measured 1e-7 .. 7e-6 at 32^3 .. 128^3)."""
    c = cases.tgv_viscous_curvilinear(128)
    P = c["params"]
    X, Y, Z = c["x"], c["y"], c["z"]
    Q0 = c["Q"].copy()
    Q0[0][I[1:]] = (1 + 0.05 * np.sin(X + 2 * Y + 3 * Z))[I[1:]]
    Q0[1][I[1:]] += 0.03
    Q0[3][I[1:]] += (0.05 + 0.02 * np.cos(2 * X - Y + Z))[I[1:]]
    Q0[5][I[1:]] = Q0[4][I[1:]] / (Q0[0][I[1:]] * P.rg)
    m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
    s = Flame3D(P)
    md, Jd = [dev(a) for a in m], dev(J)
    s.set_metrics(md, Jd)
    dU = _interior_random(U.shape, 5) * 1e-3 * np.abs(U[I]).max()
    Lb = _interior_random(U.shape, 6)
    _, jvp = orc.rhs_jvp_u(P, U, dU, m, J)
    vjp = host(s.rhs_vjp(dev(U), dev(Lb)))
    lhs, rhs = float((vjp[I] * dU[I]).sum()), float((Lb[I] * jvp[I]).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(Lb[I] * jvp[I]).sum(), (lhs, rhs)
    _, jvp = orc.rk3_jvp_u(P, 1, c["dt"], U, dU, m, J)
    g = host(s.rk3_step_vjp(c["dt"], dev(U), dev(Lb)))
    lhs, rhs = float((g[I] * dU[I]).sum()), float((Lb[I] * jvp[I]).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(Lb[I] * jvp[I]).sum(), (lhs, rhs)
    s.close()

"""Synthetic flow cases: grids with ghost coordinates and initial primitive states.

Arrays are numpy float64 in the reference layout as C-ordered (nvar, Nz+8, Ny+8, Nx+8)
(equivalently Julia (Nx+8, Ny+8, Nz+8, nvar)). Only interior cells of Q are set; the ghost
layers come from the solver's ghost fill. There is no public dataset behind any case: all
inputs are analytic fields plus seeded noise.

  tgv(n)  Taylor-Green vortex on [0, 2pi)^3, all periodic, Mach 0.1, WENO5 everywhere.
  sod(...) Sod shock tube on a sinusoidally perturbed curvilinear grid on the unit cube,
           hybrid UP7/WENO7/WENO5/NND with the shock sensor, zero-gradient x, periodic y, z.
  compression_ramp(...) viscous Mach 2.9 flow over a 24-degree ramp on a body-fitted grid,
           1/7-power-law inflow with Crocco-Busemann temperature, isothermal wall.
"""
from __future__ import annotations

import numpy as np

from .abi import (BC_DIRICHLET, BC_INFLOW_PROFILE, BC_PERIODIC, BC_WALL_ISOTHERMAL, BC_ZERO_GRADIENT, F3DParams,
                  make_params)

NG = 4


def _axis(n: int, h: float, origin: float = 0.0) -> np.ndarray:
    """Cell-centre coordinate of every full-grid index (ghosts continue the spacing)."""
    return origin + (np.arange(n + 2 * NG) - NG + 0.5) * h


def _grid3(n3):
    nx, ny, nz = n3
    return (nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)


def _interior(a: np.ndarray) -> np.ndarray:
    return a[..., NG:-NG, NG:-NG, NG:-NG]


def tgv(n: int = 64, mach: float = 0.1, gamma: float = 1.4, rg: float = 287.0, character: int = 0,
        viscous: int = 0, split: str = "SW") -> dict:
    """Inviscid Taylor-Green vortex, n^3 interior cells on [0, 2pi)^3.

    rho0 = 1, c0 = 1 (p0 = rho0 c0^2 / gamma), U0 = mach * c0; u = U0 sin x cos y cos z,
    v = -U0 cos x sin y cos z, w = 0, p = p0 + rho0 U0^2 / 16 (cos 2x + cos 2y)(cos 2z + 2),
    T = p / (rho Rg). WENO5 everywhere: phi1 = phi2 = 0, phi3 = +inf.
    """
    h = 2 * np.pi / n
    ax = _axis(n, h)
    z3, y3, x3 = np.meshgrid(ax, ax, ax, indexing="ij")
    shape = _grid3((n, n, n))
    rho0, c0 = 1.0, 1.0
    p0 = rho0 * c0 ** 2 / gamma
    U0 = mach * c0
    Q = np.zeros((6, *shape))
    Q[0] = rho0
    Q[1] = U0 * np.sin(x3) * np.cos(y3) * np.cos(z3)
    Q[2] = -U0 * np.cos(x3) * np.sin(y3) * np.cos(z3)
    Q[3] = 0.0
    Q[4] = p0 + rho0 * U0 ** 2 / 16.0 * (np.cos(2 * x3) + np.cos(2 * y3)) * (np.cos(2 * z3) + 2.0)
    Q[5] = Q[4] / (Q[0] * rg)
    Q[:, :NG] = 0; Q[:, -NG:] = 0; Q[:, :, :NG] = 0; Q[:, :, -NG:] = 0; Q[..., :NG] = 0; Q[..., -NG:] = 0
    per = dict(kind=BC_PERIODIC)
    params = make_params(n, n, n, gamma=gamma, rg=rg, phi1=0.0, phi2=0.0, phi3=float("inf"), character=character,
                         viscous=viscous, split=split, bc=[per] * 6)
    c = np.sqrt(gamma * _interior(Q[4]) / _interior(Q[0]))
    dt = 0.5 * h / float(np.abs(_interior(Q[1:4])).max() + c.max())
    return dict(name=f"tgv{n}", params=params, x=x3, y=y3, z=z3, Q=Q, dt=dt, cfl=0.5)


def tgv_viscous_curvilinear(n: int = 128, amp: float = 0.05, re: float = 1600.0, mach: float = 0.1,
                            gamma: float = 1.4, rg: float = 287.0, character: int = 0) -> dict:
    """Viscous Taylor-Green vortex on a sinusoidally perturbed periodic grid.

    x = xi + amp sin(eta) sin(zeta) and cyclic on [0, 2pi)^3 (periodic metrics), the TGV
    field of tgv(), Re = rho0 U0 L / mu0 with L = 1, the reference's Sutherland law with its
    T_s = 110.4 and C_s chosen so that mu(T0) = mu0 (the reference's SI constants would give
    another Reynolds number at this nondimensional temperature), Pr = 0.72, hybrid
    thresholds of run.jl, component-wise reconstruction by default.
    """
    c = tgv(n, mach=mach, gamma=gamma, rg=rg, character=character, viscous=1)
    P = c["params"]
    X, Y, Z = c["x"], c["y"], c["z"]
    c["x"] = X + amp * np.sin(Y) * np.sin(Z)
    c["y"] = Y + amp * np.sin(Z) * np.sin(X)
    c["z"] = Z + amp * np.sin(X) * np.sin(Y)
    rho0, c0 = 1.0, 1.0
    U0 = mach * c0
    p0 = rho0 * c0 ** 2 / gamma
    T0 = p0 / (rho0 * rg)
    mu0 = rho0 * U0 * 1.0 / re
    P.t_s = 110.4
    P.c_s = mu0 * (T0 + P.t_s) / T0 ** 1.5
    P.phi1, P.phi2, P.phi3 = 0.05, 1.0, 10.0
    c["name"] = f"tgv{n}_viscous_curvi"
    c["dt"] = c["dt"] * (1 - 2 * amp)
    return c


def sod(nx: int = 256, ny: int = 64, nz: int = 64, amp: float = 0.02, noise: float = 1e-3, seed: int = 20240601,
        gamma: float = 1.4, rg: float = 287.0, cfl: float = 0.5, character: int = 1, split: str = "SW") -> dict:
    """Sod tube on x = xi + a sin(2 pi eta) sin(2 pi zeta) (and cyclic for y, z), unit cube.

    Left (x < 0.5): rho = 1, p = 1; right: rho = 0.125, p = 0.1; at rest; uniform noise of
    amplitude `noise` on rho from numpy's PCG64 with `seed`. Hybrid thresholds of run.jl
    (0.05, 1, 10), inviscid, zero-gradient in x and periodic in y, z. The coordinates are
    the analytic map evaluated at every cell including ghosts (periodic in y and z).
    """
    xi, eta, zeta = _axis(nx, 1.0 / nx), _axis(ny, 1.0 / ny), _axis(nz, 1.0 / nz)
    Z, E, X = np.meshgrid(zeta, eta, xi, indexing="ij")
    tp = 2 * np.pi
    x3 = X + amp * np.sin(tp * E) * np.sin(tp * Z)
    y3 = E + amp * np.sin(tp * Z) * np.sin(tp * X)
    z3 = Z + amp * np.sin(tp * X) * np.sin(tp * E)
    shape = _grid3((nx, ny, nz))
    rng = np.random.default_rng(seed)
    left = x3 < 0.5
    Q = np.zeros((6, *shape))
    Q[0] = np.where(left, 1.0, 0.125) + noise * rng.uniform(-1.0, 1.0, size=shape)
    Q[4] = np.where(left, 1.0, 0.1)
    Q[5] = Q[4] / (Q[0] * rg)
    for a in Q:
        a[:NG] = 0; a[-NG:] = 0; a[:, :NG] = 0; a[:, -NG:] = 0; a[..., :NG] = 0; a[..., -NG:] = 0
    zg, per = dict(kind=BC_ZERO_GRADIENT), dict(kind=BC_PERIODIC)
    params = make_params(nx, ny, nz, gamma=gamma, rg=rg, character=character, viscous=0, split=split,
                         bc=[zg, zg, per, per, per, per])
    cmax = np.sqrt(gamma * 1.0 / (1.0 - noise))
    dt = cfl * (1.0 - 2 * amp * tp) / max(nx, ny, nz) / cmax
    return dict(name=f"sod{nx}x{ny}x{nz}", params=params, x=x3, y=y3, z=z3, Q=Q, dt=dt, cfl=cfl)


def compression_ramp(nx: int = 512, ny: int = 256, nz: int = 128, angle_deg: float = 24.0, mach: float = 2.9,
                     re: float = 1e5, first_cell: float = 1e-3, x_up: float = 8.0, x_down: float = 8.0,
                     height: float = 10.0, span: float = 4.0, gamma: float = 1.4, rg: float = 287.0,
                     pr: float = 0.72, t_inf_kelvin: float = 108.1, character: int = 1, cfl: float = 0.5) -> dict:
    """Viscous supersonic flow over a compression ramp (streamwise x wall-normal x spanwise).

    Lengths in inflow boundary-layer thicknesses delta; rho_inf = 1, c_inf = 1, so
    p_inf = 1/gamma, U_inf = mach, T_inf = p_inf/(rho_inf Rg) with the reference's Rg.
    Re = rho_inf U_inf delta / mu_inf. Sutherland's law with T_s = T_inf * 110.4 K /
    t_inf_kelvin (the ratio of a Mach 2.9 tunnel at t_inf_kelvin static temperature) and
    C_s set so that mu(T_inf) = mu_inf; Pr = 0.72. Grid: grid.compression_ramp_grid (tanh
    wall-normal stretching, first cell `first_cell` delta at the inflow; spanwise periodic).
    Inflow (x- face, per point): u = U_inf (d/delta)^(1/7) for wall distance d < delta, with
    the Crocco-Busemann temperature T = T_w + (T_aw - T_w) u/U - (T_aw - T_inf) (u/U)^2,
    T_w = T_aw = T_inf (1 + r (gamma-1)/2 M^2), r = Pr^(1/3); p = p_inf; rho = p/(Rg T).
    Walls: isothermal at T_w (y-); freestream Dirichlet on top (y+), as boundary.jl:96-118;
    zero-gradient outflow (x+, boundary.jl:42-51); periodic in z. Initial field: the inflow
    profile by vertical wall distance at every station, flow along x. Hybrid thresholds of
    run.jl, Steger-Warming, viscous.
    Returns the usual case dict plus `profile` ((5, Nz+8, Ny+8), face 0) and `wall`
    (T_w, mu_w, U_inf, rho_inf, p_inf) for wall quantities.
    """
    from .grid import compression_ramp_grid, ramp_wall
    x, y, z, beta = compression_ramp_grid(nx, ny, nz, angle_deg, x_up, x_down, height, span, first_cell)
    rho_inf, c_inf = 1.0, 1.0
    p_inf = rho_inf * c_inf ** 2 / gamma
    u_inf = mach * c_inf
    t_inf = p_inf / (rho_inf * rg)
    mu_inf = rho_inf * u_inf * 1.0 / re
    t_s = t_inf * 110.4 / t_inf_kelvin
    c_s = mu_inf * (t_inf + t_s) / t_inf ** 1.5
    r = pr ** (1.0 / 3.0)
    t_aw = t_inf * (1.0 + r * 0.5 * (gamma - 1.0) * mach ** 2)
    t_w = t_aw
    mu_w = c_s * t_w ** 1.5 / (t_w + t_s)

    def state(d):
        f = np.clip(d, 0.0, None) ** (1.0 / 7.0)
        f = np.where(d >= 1.0, 1.0, f)
        T = t_w + (t_aw - t_w) * f - (t_aw - t_inf) * f ** 2
        rho = p_inf / (rg * T)
        return rho, u_inf * f, T

    nzt, nyt, nxt = x.shape
    shape = (nzt, nyt, nxt)
    d = y - ramp_wall(x, angle_deg, 0.5)
    rho, u, T = state(d)
    Q = np.zeros((6, *shape))
    Q[0], Q[1], Q[4], Q[5] = rho, u, p_inf, T
    for a in Q:
        a[:NG] = 0; a[-NG:] = 0; a[:, :NG] = 0; a[:, -NG:] = 0; a[..., :NG] = 0; a[..., -NG:] = 0
    # inflow profile over the full (k, j) extent of the x- face, from the first interior column
    d0 = y[:, :, NG] - ramp_wall(x[:, :, NG], angle_deg, 0.5)
    rho0, u0, _ = state(d0)
    prof = np.zeros((5, nzt, nyt))
    prof[0], prof[1], prof[4] = rho0, u0, p_inf
    fs = dict(kind=BC_DIRICHLET, rho=rho_inf, u=u_inf, v=0.0, w=0.0, p=p_inf)
    params = make_params(nx, ny, nz, gamma=gamma, rg=rg, pr=pr, c_s=c_s, t_s=t_s, character=character, viscous=1,
                         split="SW", bc=[dict(kind=BC_INFLOW_PROFILE), dict(kind=BC_ZERO_GRADIENT),
                                         dict(kind=BC_WALL_ISOTHERMAL, t_wall=t_w), fs,
                                         dict(kind=BC_PERIODIC), dict(kind=BC_PERIODIC)])
    # time step: the smallest grid spacing (first cell, sheared by the ramp) against the
    # fastest signal (U_inf plus the sound speed at the wall temperature)
    dx = (x_up + x_down) / nx
    dy1 = float((y[NG:-NG, NG + 1, NG:-NG] - y[NG:-NG, NG, NG:-NG]).min())
    smax = u_inf + c_inf * np.sqrt(t_w / t_inf)
    dt = cfl * min(dx, dy1 * np.cos(np.radians(angle_deg)), span / nz) / smax
    return dict(name=f"ramp{nx}x{ny}x{nz}", params=params, x=x, y=y, z=z, Q=Q, dt=dt, cfl=cfl, profile=prof,
                wall=dict(t_w=t_w, mu_w=mu_w, u_inf=u_inf, rho_inf=rho_inf, p_inf=p_inf, beta=beta,
                          angle_deg=angle_deg))


def interior(a: np.ndarray) -> np.ndarray:
    return _interior(a)


def params_copy(p: F3DParams, **kw) -> F3DParams:
    """Copy of p with scalar fields overridden."""
    import ctypes
    q = F3DParams()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(F3DParams))
    for k, v in kw.items():
        setattr(q, k, v)
    return q

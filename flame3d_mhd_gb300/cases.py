"""Synthetic flow cases: grids with ghost coordinates and initial primitive states.

Arrays are numpy float64 in the reference layout as C-ordered (nvar, Nz+8, Ny+8, Nx+8)
(equivalently Julia (Nx+8, Ny+8, Nz+8, nvar)). Only interior cells of Q are set; the ghost
layers come from the solver's ghost fill. There is no public dataset behind any case: all
inputs are analytic fields plus seeded noise.

  tgv(n)  Taylor-Green vortex on [0, 2pi)^3, all periodic, Mach 0.1, WENO5 everywhere.
  sod(...) Sod shock tube on a sinusoidally perturbed curvilinear grid on the unit cube,
           hybrid UP7/WENO7/WENO5/NND with the shock sensor, zero-gradient x, periodic y, z.
"""
from __future__ import annotations

import numpy as np

from .abi import (BC_PERIODIC, BC_ZERO_GRADIENT, F3DParams, make_params)

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

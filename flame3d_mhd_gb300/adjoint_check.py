"""Gradient check of the discrete adjoint on the viscous curvilinear Taylor-Green vortex.

  python -m flame3d_mhd_gb300.adjoint_check --n 128 --steps 400 --dirs 8

J(U0) = volume-integrated kinetic energy after N SSP-RK3 steps (128^3, curvilinear amplitude
0.05, Re 1600, Mach 0.1, FP64, component-wise hybrid). dJ/dU0 comes from ceil(sqrt(N))
checkpoints and step VJPs (f3d_rk3_step_vjp); each of `dirs` seeded Gaussian directions d
(entries N(0, 1) scaled per variable by max |U| over the interior; --normalise divides each by
its L2 norm, which shrinks every entry ~3e3-fold at 128^3 and leaves the difference of the two
J values below FP64 rounding of the 400-step trajectories) is checked against the central
difference (J(U0 + h d) - J(U0 - h d)) / 2h with h = 1e-6. Prints one JSON line with, per
direction, the adjoint and difference values and their relative difference, and the times of
the forward pass and of the gradient.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np
import torch

from . import cases
from .adjoint import backward_from_checkpoints, forward_with_checkpoints
from .solver import Flame3D

NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def kinetic_energy(U: torch.Tensor, vol: torch.Tensor) -> float:
    r = U[I][0]
    ke = 0.5 * (U[I][1] ** 2 + U[I][2] ** 2 + U[I][3] ** 2) / r
    return float((ke * vol).sum())


def kinetic_energy_grad(U: torch.Tensor, vol: torch.Tensor) -> torch.Tensor:
    g = torch.zeros_like(U)
    r = U[I][0]
    m2 = U[I][1] ** 2 + U[I][2] ** 2 + U[I][3] ** 2
    g[0][I[1:]] = -0.5 * m2 / r ** 2 * vol
    for k in (1, 2, 3):
        g[k][I[1:]] = U[I][k] / r * vol
    return g


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--dirs", type=int, default=8)
    ap.add_argument("--h", type=str, default="1e-6",
                    help="difference step(s), comma-separated: the error of a central difference falls "
                         "as h^2 until the rounding of J (about 1e-16 J / h) takes over")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--normalise", action="store_true", help="unit L2 norm directions")
    ap.add_argument("--character", type=int, default=0, help="1: characteristic-wise reconstruction")
    ap.add_argument("--generic", action="store_true",
                    help="add smooth 3-D variations of rho, w, p and a drift to the vortex: its symmetry "
                         "otherwise puts contravariant velocities exactly on the Steger-Warming kink, "
                         "where the derivative is one-sided")
    a = ap.parse_args(argv)
    c = cases.tgv_viscous_curvilinear(a.n)
    P = c["params"]
    P.character = a.character
    if a.generic:
        X, Y, Z, Ii = c["x"], c["y"], c["z"], I[1:]
        Qg = c["Q"].copy()
        Qg[0][Ii] = (1 + 0.05 * np.sin(X + 2 * Y + 3 * Z))[Ii]
        Qg[1][Ii] += 0.03
        Qg[2][Ii] += 0.02
        Qg[3][Ii] += (0.05 + 0.02 * np.cos(2 * X - Y + Z))[Ii]
        Qg[4][Ii] *= (1 + 0.03 * np.cos(3 * X + Y - 2 * Z))[Ii]
        Qg[5][Ii] = Qg[4][Ii] / (Qg[0][Ii] * P.rg)
        c["Q"] = Qg
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    s = Flame3D(P)
    ms, J = s.compute_metrics(dev(c["x"]), dev(c["y"]), dev(c["z"]))
    s.set_metrics(ms, J)
    vol = 1.0 / J[I[1:]]
    Q = dev(c["Q"])
    U0 = s.field(5)
    s.prim2c(U0, Q)
    s.fillGhost(Q, U0)
    dt, N = c["dt"], a.steps

    def J_of(Ustart: torch.Tensor) -> float:
        U = Ustart.clone()
        Un, Qs = s.field(5), s.field(6)
        s.q_from_u(U, Qs)
        s.time_step(U, Un, Qs, dt, N)
        return kinetic_energy(U, vol)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    UN, ckpt, every = forward_with_checkpoints(s, U0, dt, N)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    grad = backward_from_checkpoints(s, ckpt, every, dt, N, kinetic_energy_grad(UN, vol))
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    J0 = kinetic_energy(UN, vol)
    rng = np.random.default_rng(a.seed)
    rows = []
    scale = U0[I].abs().amax(dim=(1, 2, 3)).cpu().numpy()
    for k in range(a.dirs):
        d = np.zeros(tuple(U0.shape))
        d[I] = rng.standard_normal(d[I].shape) * scale[:, None, None, None]
        if a.normalise:
            d /= np.linalg.norm(d)
        dd = dev(d)
        ad = float((grad * dd).sum())
        for h in [float(v) for v in a.h.split(",")]:
            fd = (J_of(U0 + h * dd) - J_of(U0 - h * dd)) / (2 * h)
            rows.append({"dir": k, "h": h, "adjoint": ad, "central_difference": fd, "rel_diff": abs(fd - ad) / abs(ad)})
    mode = "characteristic" if a.character else "component-wise"
    out = {"case": f"tgv{a.n}^3 viscous curvilinear (amp 0.05, Re 1600, Mach 0.1), FP64, {mode} hybrid"
                   + (", with smooth variations and drift" if a.generic else ""),
           "directions_kind": "seeded Gaussian, per-variable scaled by max|U|"
                              + (", unit L2 norm" if a.normalise else ", not normalised"),
           "steps": N, "dt": dt, "checkpoint_every": every, "checkpoints": len(ckpt), "J": J0,
           "forward_s": t1 - t0, "gradient_s": t2 - t1,
           "max_rel_diff_per_h": {str(h): max(r["rel_diff"] for r in rows if r["h"] == h)
                                  for h in sorted({r["h"] for r in rows})},
           "directions": rows}
    print(json.dumps(out))
    s.close()
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)

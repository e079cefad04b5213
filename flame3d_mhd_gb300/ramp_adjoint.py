"""Compression ramp: a mixed-precision forward run and the discrete adjoint of the wall
pressure force over the last steps with respect to the inflow profile and the ramp angle.

  python -m flame3d_mhd_gb300.ramp_adjoint --nx 1024 --ny 384 --nz 192 --steps 1000 --window 200

Objective: J = dt * sum over the last `window` states U_n (n = N - window + 1 .. N) of a
component of the wall-pressure force, the pressure of the first cell layer times the wall
faces' area vectors (the J^-1-scaled eta metrics, grad eta pointing into the fluid, so the
force on the wall is -p J^-1 grad eta):
  --force y (default): the wall load, F = sum_{i,k} p(U_n)[i, 0, k] (J^-1 eta_y)[i, 0, k];
  --force x: the drag on the ramp, F = -sum_{i,k} p(U_n)[i, 0, k] (J^-1 eta_x)[i, 0, k] (on
    the flat wall upstream eta_x = 0, so within the first steps the inflow reaches no part
    of it). Parameters:
  - s, the wall-normal vector of inflow velocity scalings: the inflow profile's u at
    wall-normal row j is s_j u_0(j) (s = 1 nominal; one entry per interior row);
  - theta, the ramp angle in degrees, through the grid (compression_ramp_grid) and so the
    metrics and Jacobian of every cell; the initial state and the inflow profile are the
    nominal ones at every theta.
Gradients (FP64 state, component-wise hybrid reconstruction, Steger-Warming):
  - dJ/ds from the adjoint: the step VJPs carry the ghost cotangents of the inflow face into
    the profile (f3d_set_inflow_profile_cotangent), dJ/ds_j = sum_k profile_bar[u, k, j] u_0;
  - dJ/dtheta (--angle-method adjoint, the default) = <metrics_bar, dm/dtheta> + <J_bar,
    dJ/dtheta> + the objective's own area term: the step VJPs accumulate the cotangents of
    the nine metrics and J (f3d_set_metrics_cotangent), and the metrics' derivative in theta
    is a central difference of the grid generator and the metric kernel over theta +- eta
    (once, not per step). --angle-method fd instead forms sum over steps and stages
    <Lbar_s, dL/dtheta at V_s> from the stage states V_s and RHS cotangents Lbar_s of every
    step VJP (f3d_rk3_step_vjp_stages), with dL/dtheta at fixed V_s a central difference of
    the RHS over the two metric sets (6 RHS per step): an independent check of the first.
The reversal holds at most `slots` trajectory states, sized from the memory left under
`--hbm-gb` after the solver contexts (multi-level checkpointing, adjoint.plan).
Checks: central differences of J in FP64 along seeded unit directions of s and in theta.
The mixed-precision forward run (FP32 fluxes, FP64 state) of the same case is timed and its
J compared with the FP64 one.

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np
import torch

from . import cases
from .abi import PREC_MIXED
from .adjoint import plan, trajectory_gradient
from .cases import params_copy
from .grid import compression_ramp_grid
from .solver import Flame3D, side_stream

NG = 4


def pressure(U: torch.Tensor, gamma: float) -> torch.Tensor:
    """p of the first interior cell layer above the eta = 0 wall, (Nz, Nx)."""
    u = U[:, NG:-NG, NG, NG:-NG]
    return (gamma - 1.0) * (u[4] - 0.5 * (u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / u[0])


def pressure_grad(U: torch.Tensor, gamma: float, w: torch.Tensor) -> torch.Tensor:
    """Cotangent of U for the scalar sum(w * p) over the first cell layer."""
    g = torch.zeros_like(U)
    u = U[:, NG:-NG, NG, NG:-NG]
    r = u[0]
    gm = gamma - 1.0
    g[0, NG:-NG, NG, NG:-NG] = w * gm * 0.5 * (u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / r ** 2
    for k in (1, 2, 3):
        g[k, NG:-NG, NG, NG:-NG] = -w * gm * u[k] / r
    g[4, NG:-NG, NG, NG:-NG] = w * gm
    return g


class RampAdjoint:
    """The FP64 ramp context, its objective and gradients."""

    def __init__(self, a, dev: str = "cuda"):
        self.a = a
        self.case = cases.compression_ramp(a.nx, a.ny, a.nz, angle_deg=a.angle, first_cell=a.first_cell,
                                           character=0)
        if a.branch == "weno5":  # thresholds that leave the sensor no choice: WENO5 at every face
            self.case["params"] = params_copy(self.case["params"], phi1=0.0, phi2=0.0, phi3=5.0)
        # one prepared stage state in the step VJP: 16 grid-sized arrays more for trajectory states
        self.case["params"] = params_copy(self.case["params"], adjoint_lean=1)
        P = self.case["params"]
        self.gamma = P.gamma
        self.to = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
        self.s = Flame3D(P)
        self.metrics = {0: self._metrics(a.angle)}
        self.s.set_metrics(*self.metrics[0])
        self.prof0 = self.to(self.case["profile"])
        self.prof = self.prof0.clone()
        self.s.set_inflow_profile(0, self.prof)
        Q = self.to(self.case["Q"])
        self.U0 = self.s.field(5)
        self.s.prim2c(self.U0, Q)
        self.s.fillGhost(Q, self.U0)
        self.dt, self.N, self.W = self.case["dt"], a.steps, a.window
        self.rows = slice(NG, NG + a.ny)

    def _metrics(self, angle: float):
        x, y, z, _ = compression_ramp_grid(self.a.nx, self.a.ny, self.a.nz, angle, first_cell=self.a.first_cell)
        ms, J = self.s.compute_metrics(self.to(x), self.to(y), self.to(z))
        return ms, J

    def area(self, metrics) -> torch.Tensor:
        """Weights of the first-layer pressures in the force component, (Nz, Nx)."""
        if self.a.force == "x":
            return -metrics[0][3][NG:-NG, NG, NG:-NG]
        return metrics[0][4][NG:-NG, NG, NG:-NG]

    def objective(self, U_of_n, n: int, acc: list, area: torch.Tensor):
        if n > self.N - self.W:
            acc.append(self.dt * (pressure(U_of_n, self.gamma) * area).sum())

    def set_scaling(self, scale: torch.Tensor | None):
        self.prof.copy_(self.prof0)
        if scale is not None:
            self.prof[1, :, self.rows] *= scale[None, :]

    def J(self, metrics=None) -> float:
        """FP64 forward run of N steps from the nominal initial state; J of the window."""
        m = metrics or self.metrics[0]
        if metrics is not None:
            self.s.set_metrics(*m)
        area = self.area(m)
        acc = []
        U = self.U0.clone()
        Un, Q = self.s.field(5), self.s.field(6)
        with side_stream():
            self.s.q_from_u(U, Q)
            for n in range(1, self.N + 1):
                self.s.time_step(U, Un, Q, self.dt, 1)
                self.objective(U, n, acc, area)
        val = float(torch.stack(acc).sum())
        if metrics is not None:
            self.s.set_metrics(*self.metrics[0])
        return val


def mixed_forward(R: "RampAdjoint", cells: int, J0: float, area0: torch.Tensor) -> dict:
    """The same N steps in mixed precision (FP32 fluxes, FP64 state): time per step of the
    steps before the window and J of the window, against the FP64 J0."""
    Pm = params_copy(R.case["params"], precision=PREC_MIXED, adjoint_lean=0)
    sm = Flame3D(Pm)
    sm.set_metrics(*R.metrics[0])
    sm.set_inflow_profile(0, R.prof0)
    U, Un, Q = R.U0.clone(), sm.field(5), sm.field(6)
    acc = []
    with side_stream() as stream:
        sm.q_from_u(U, Q)
        sm.time_step(U, Un, Q, R.dt, 1)  # capture the step graph
        R.objective(U, 1, acc, area0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sm.time_step(U, Un, Q, R.dt, R.N - R.W - 1)
        e1.record(stream)
        for n in range(R.N - R.W + 1, R.N + 1):
            sm.time_step(U, Un, Q, R.dt, 1)
            R.objective(U, n, acc, area0)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(R.N - R.W - 1, 1)
    Jm = float(torch.stack(acc).sum())
    sm.close()
    return {"ms_per_step": ms, "mcell_rhs_per_s": 3 * cells / (ms * 1e3), "J": Jm,
            "J_rel_diff_vs_fp64": abs(Jm - J0) / abs(J0)}



def progress(what: str, obj) -> None:
    """One JSON line on stderr as each part of a long run completes (the full result is
    printed on stdout at the end)."""
    print(json.dumps({"progress": what, **({"out": obj} if not isinstance(obj, dict) else obj)}),
          file=sys.stderr, flush=True)

def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--ny", type=int, default=384)
    ap.add_argument("--nz", type=int, default=192)
    ap.add_argument("--angle", type=float, default=24.0)
    ap.add_argument("--first-cell", type=float, default=1e-3)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--window", type=int, default=200)
    ap.add_argument("--force", choices=("x", "y"), default="y", help="force component of the objective")
    ap.add_argument("--branch", choices=("hybrid", "weno5"), default="hybrid",
                    help="hybrid: the sensor switches UP7 / WENO7 / WENO5 per face (J is then piecewise "
                         "smooth in the parameters); weno5: one reconstruction everywhere")
    ap.add_argument("--hbm-gb", type=float, default=180.0, help="memory budget of the whole run")
    ap.add_argument("--slots", type=int, default=0, help="trajectory states held (0: from --hbm-gb)")
    ap.add_argument("--angle-method", choices=("adjoint", "fd"), default="adjoint",
                    help="adjoint: metric and Jacobian cotangents from the VJP kernels, dotted with the metrics' "
                         "derivative in theta; fd: per stage, a central difference of the RHS over the metric "
                         "sets at theta +- eta (6 RHS per step)")
    ap.add_argument("--eta", type=float, default=1e-3,
                    help="angle step (degrees) of the metrics' (adjoint) or the RHS's (fd) difference in theta")
    ap.add_argument("--fd-dirs", type=int, default=1, help="seeded directions of s checked by central differences")
    ap.add_argument("--fd-h", type=str, default="1e-6", help="difference step(s) of s (comma-separated)")
    ap.add_argument("--fd-angle-h", type=str, default="1e-3", help="difference step(s) of theta in degrees")
    ap.add_argument("--mixed", type=int, default=1, help="also time the mixed-precision forward run")
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--forward-only", action="store_true",
                    help="only the FP64 and mixed-precision forward runs and their J (no adjoint)")
    ap.add_argument("--fd-only", action="store_true",
                    help="only J and its central differences in theta (no adjoint, no mixed run): the "
                         "difference's dependence on h separates truncation (h^2) from kinks of the "
                         "scheme crossed between theta - h and theta + h (h)")
    a = ap.parse_args(argv)
    torch.cuda.init()
    R = RampAdjoint(a)
    s, cells = R.s, a.nx * a.ny * a.nz
    out = {"case": R.case["name"] + (", component-wise hybrid WENO, SW" if a.branch == "hybrid" else
                                     ", component-wise WENO5, SW"), "steps": a.steps, "window": a.window,
           "objective": f"dt * sum of the wall-pressure force ({a.force}) over the last {a.window} states",
           "dt": R.dt, "cells": cells}

    # metric sets at theta +- eta for the RHS difference (swapped into the context for it)
    mp, mm = R._metrics(a.angle + a.eta), R._metrics(a.angle - a.eta)
    dA = (R.area(mp) - R.area(mm)) / (2 * a.eta)

    if a.forward_only:  # J in FP64 and the mixed-precision forward run, no gradient
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J0 = R.J()
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        out["fp64_forward"] = {"s": t_fwd, "mcell_rhs_per_s": 3 * cells * a.steps / t_fwd / 1e6}
        out["J"] = J0
        out["mixed_forward"] = mixed_forward(R, cells, J0, R.area(R.metrics[0]))
        print(json.dumps(out))
        s.close()
        return out
    if a.fd_only:
        out["J"] = R.J()
        out["checks"] = []
        for h in [float(v) for v in a.fd_angle_h.split(",") if v]:
            fd = (R.J(R._metrics(a.angle + h)) - R.J(R._metrics(a.angle - h))) / (2 * h)
            out["checks"].append({"param": "theta_deg", "h": h, "central_difference": fd})
        print(json.dumps(out))
        s.close()
        return out
    # allocate the context's adjoint scratch (first VJP call) and capture the step graph
    s.rk3_step_vjp(R.dt, R.U0, torch.zeros_like(R.U0))
    # FP64 forward run (the cost yardstick and J)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J0 = R.J()
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    out["fp64_forward"] = {"s": t_fwd, "mcell_rhs_per_s": 3 * cells * a.steps / t_fwd / 1e6}
    out["J"] = J0
    progress("fp64_forward", out)

    # memory: slots of one state each
    state_b = R.U0.numel() * 8
    used = None
    if a.slots > 0:
        slots = a.slots
    else:
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        free, total = torch.cuda.mem_get_info()
        used = total - free
        # stage states and cotangents (6), the reversal's Un, Q (6/5) and step scratch, the
        # cotangent, the final state, the two RHS buffers of the angle term, the objective's
        # source term, the angle term's Q and the forward pass's Un, Q: 19 states of headroom
        reserve = 19 * state_b
        slots = int((a.hbm_gb * 1e9 - used - reserve) // state_b)
        if slots < 2:
            raise SystemExit(f"--hbm-gb {a.hbm_gb} leaves no room for trajectory states ({used / 1e9:.1f} GB used)")
    out["memory"] = {"state_gb": state_b / 1e9, "slots": slots, "plan": plan(a.steps, slots),
                     "budget_gb": a.hbm_gb, "used_before_reversal_gb": None if used is None else used / 1e9}

    pbar = torch.zeros_like(R.prof)
    s.set_inflow_profile_cotangent(0, pbar)
    area0 = R.area(R.metrics[0])
    theta = {"stages": torch.zeros((), dtype=torch.float64, device=R.U0.device),
             "area": torch.zeros((), dtype=torch.float64, device=R.U0.device)}
    Qs, Lp, Lm = s.field(6), s.field(5), s.field(5)

    def observe(n, U):
        if n > R.N - R.W:
            theta["area"] += R.dt * (pressure(U, R.gamma) * dA).sum()

    def source(n, U):
        if n > R.N - R.W:
            return pressure_grad(U, R.gamma, R.dt * area0)
        return None

    sink_s = [0.0]

    def stage_sink(n, Ust, Lbt):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for k in range(3):
            s.q_from_u(Ust[k], Qs)
            s.set_metrics(*mp)
            s.rhs(Qs, Lp)
            s.set_metrics(*mm)
            s.rhs(Qs, Lm)
            Lp.sub_(Lm)  # the RHS is written at interior cells; Lbar_s is zero at ghost cells
            theta["stages"] += torch.dot(Lbt[k].view(-1), Lp.view(-1)) / (2 * a.eta)
        s.set_metrics(*R.metrics[0])
        torch.cuda.synchronize()
        sink_s[0] += time.perf_counter() - t

    mbar = Jbar = None
    if a.angle_method == "adjoint":  # metric and Jacobian cotangents accumulated by the VJPs
        mbar, Jbar = [s.field(1) for _ in range(9)], s.field(1)
        s.set_metrics_cotangent(mbar, Jbar)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with side_stream():
        UN, U0bar, st = trajectory_gradient(s, R.U0, R.dt, R.N, slots, final_grad=lambda U: source(R.N, U),
                                            source=source, observe=observe,
                                            stage_sink=stage_sink if a.angle_method == "fd" else None)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    out["reversal"] = st
    del UN, U0bar
    out["memory"]["peak_allocated_gb"] = torch.cuda.max_memory_allocated() / 1e9
    s.set_inflow_profile_cotangent(0, None)
    if mbar is not None:
        # dJ/dtheta = <metrics-bar, dm/dtheta> + <J-bar, dJ/dtheta>, the metric derivatives by
        # a central difference of the grid generator and the metric kernel over +- eta
        s.set_metrics_cotangent(None)
        for k in range(9):
            theta["stages"] += torch.dot(mbar[k].view(-1), ((mp[0][k] - mm[0][k]) / (2 * a.eta)).view(-1))
        theta["stages"] += torch.dot(Jbar.view(-1), ((mp[1] - mm[1]) / (2 * a.eta)).view(-1))
        del mbar, Jbar
    u0 = R.prof0[1, :, R.rows]
    dJds = (pbar[1, :, R.rows] * u0).sum(dim=0)
    dJdtheta = float(theta["stages"] + theta["area"])
    out["gradient"] = {"dJds_norm": float(dJds.norm()), "dJds_first_rows": dJds[:4].tolist(),
                       "dJdtheta_deg": dJdtheta, "dJdtheta_area_term": float(theta["area"]),
                       "angle_method": a.angle_method}
    # the angle's stage differences (6 RHS per step) are timed apart: without them the
    # reversal is the profile (and initial-state) gradient alone
    out["cost"] = {"gradient_s": t_grad, "angle_stage_differences_s": sink_s[0],
                   "adjoint_over_forward": t_grad / t_fwd,
                   "adjoint_over_forward_without_angle": (t_grad - sink_s[0]) / t_fwd}
    progress("gradient", out)

    # central differences in FP64
    rng = np.random.default_rng(a.seed)
    checks = []
    for k in range(a.fd_dirs):
        d = torch.from_numpy(rng.standard_normal(a.ny)).to(R.U0.device)
        d /= d.norm()
        ad = float((dJds * d).sum())
        for h in [float(v) for v in a.fd_h.split(",")]:
            R.set_scaling(1.0 + h * d)
            Jp = R.J()
            R.set_scaling(1.0 - h * d)
            Jm = R.J()
            R.set_scaling(None)
            fd = (Jp - Jm) / (2 * h)
            checks.append({"param": "s", "dir": k, "h": h, "adjoint": ad, "central_difference": fd,
                           "rel_diff": abs(fd - ad) / max(abs(ad), 1e-300)})
            progress("check", checks[-1])
    for h in [float(v) for v in a.fd_angle_h.split(",") if v]:
        Jp = R.J(R._metrics(a.angle + h))
        Jm = R.J(R._metrics(a.angle - h))
        fd = (Jp - Jm) / (2 * h)
        checks.append({"param": "theta_deg", "h": h, "adjoint": dJdtheta, "central_difference": fd,
                       "rel_diff": abs(fd - dJdtheta) / max(abs(dJdtheta), 1e-300)})
    out["checks"] = checks

    if a.mixed:
        out["mixed_forward"] = mixed_forward(R, cells, J0, area0)
    out["max_rel_diff"] = max((c["rel_diff"] for c in checks), default=None)
    print(json.dumps(out))
    s.close()
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)

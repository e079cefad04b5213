"""Compression-ramp study: FP64 and mixed precision from the same initial state, compared
by wall pressure and skin friction.

  python -m flame3d_mhd_gb300.ramp --nx 512 --ny 256 --nz 128 --steps 500

prints one JSON line: the case, time per step and Mcell-RHS/s of both forms, and the
deviation of the mixed form's wall pressure and skin friction from the FP64 form's, each as
max |mixed - FP64| / max |FP64| over the wall, plus the mean-value deviations.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np
import torch

from . import cases, files
from .abi import PREC_MIXED
from .solver import Flame3D, side_stream

NG = 4


def wall_pressure(Q: np.ndarray) -> np.ndarray:
    """Pressure of the first cell layer above the eta = 0 wall, (Nz, Nx)."""
    return Q[4, NG:-NG, NG, NG:-NG]


def skin_friction(Q: np.ndarray, x: np.ndarray, y: np.ndarray, wall: dict) -> np.ndarray:
    """C_f = tau_w / (rho_inf U_inf^2 / 2), (Nz, Nx), with tau_w = mu_w du_t/dn from the
    first cell and its ghost (the no-slip mirror) across the wall face; t is the wall
    tangent along xi (centred differences of the wall-face midpoints), n its normal."""
    I = (slice(NG, -NG), slice(None), slice(NG, -NG))
    xw = 0.5 * (x[:, NG - 1, :] + x[:, NG, :])
    yw = 0.5 * (y[:, NG - 1, :] + y[:, NG, :])
    tx = np.gradient(xw, axis=1)
    ty = np.gradient(yw, axis=1)
    nrm = np.hypot(tx, ty)
    tx, ty = tx / nrm, ty / nrm
    nx_, ny_ = -ty, tx
    dist = (x[:, NG, :] - x[:, NG - 1, :]) * nx_ + (y[:, NG, :] - y[:, NG - 1, :]) * ny_
    ut1 = Q[1, :, NG, :] * tx + Q[2, :, NG, :] * ty
    utg = Q[1, :, NG - 1, :] * tx + Q[2, :, NG - 1, :] * ty
    tau = wall["mu_w"] * (ut1 - utg) / dist
    cf = tau / (0.5 * wall["rho_inf"] * wall["u_inf"] ** 2)
    return cf[I[0], I[2]]


def run(case: dict, precision: int, steps: int, dev: str = "cuda", perturb: float = 0.0,
        seed: int = 7, out_dir: str | None = None, wall_only: bool = False) -> tuple[np.ndarray, float]:
    """Advance `steps` SSP-RK3 steps (graph-captured) and return (Q, ms per step). With
    perturb > 0 the initial interior primitive state is multiplied by 1 + perturb * N(0,1)
    (seeded): an FP64 run perturbed at FP32 rounding level measures how far the flow itself
    amplifies last-bit differences (the yardstick for the mixed form's deviation).
    With `out_dir` the reference's files are written there: metrics.h5 and mesh.h5 from the
    device metrics and the grid, and after the last step PLT/plt-<steps>.h5 + .xmf and
    CHK/chk-<steps>.h5 from the primitives of the final state and their shock sensor.
    wall_only: return only the eta layers 0..NG of Q (all wall_pressure and skin_friction
    read), which keeps the host copy small on large grids."""
    from .cases import params_copy
    P = params_copy(case["params"], precision=precision)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    s = Flame3D(P)
    ms, J = s.compute_metrics(to(case["x"]), to(case["y"]), to(case["z"]))
    s.set_metrics(ms, J)
    if out_dir:
        files.write_metrics(os.path.join(out_dir, "metrics.h5"), ms, J)
        files.write_mesh(os.path.join(out_dir, "mesh.h5"), case["x"], case["y"], case["z"])
    s.set_inflow_profile(0, to(case["profile"]))
    Q0 = case["Q"]
    if perturb > 0.0:
        rng = np.random.default_rng(seed)
        Q0 = Q0 * (1.0 + perturb * rng.standard_normal(Q0.shape))
    Q = to(Q0)
    U, Un = s.field(5), s.field(5)
    s.prim2c(U, Q)
    s.fillGhost(Q, U)
    with side_stream() as stream:
        s.time_step(U, Un, Q, case["dt"], 1)  # capture the step graph
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.time_step(U, Un, Q, case["dt"], steps - 1)
        e1.record(stream)
        e1.synchronize()
    s.check_finite(U)
    out = (Q[:, :, :NG + 1, :] if wall_only else Q).cpu().numpy()
    if out_dir:
        Qf = s.q_from_u(U)
        phi = s.field(1)
        s.shockSensor(phi, Qf)
        files.plotFile_xdmf(out_dir, steps, Qf, phi, case["dt"])
        files.checkpointFile(out_dir, steps, Qf)
    s.close()
    return out, e0.elapsed_time(e1) / max(steps - 1, 1)


def deviations(Q64: np.ndarray, Q32: np.ndarray, case: dict) -> dict:
    pw64, pw32 = wall_pressure(Q64), wall_pressure(Q32)
    cf64 = skin_friction(Q64, case["x"], case["y"], case["wall"])
    cf32 = skin_friction(Q32, case["x"], case["y"], case["wall"])
    return {
        "wall_pressure_rel_linf": float(np.abs(pw32 - pw64).max() / np.abs(pw64).max()),
        "wall_pressure_mean_rel": float(abs(pw32.mean() - pw64.mean()) / abs(pw64.mean())),
        "skin_friction_rel_linf": float(np.abs(cf32 - cf64).max() / np.abs(cf64).max()),
        "skin_friction_mean_rel": float(abs(cf32.mean() - cf64.mean()) / abs(cf64.mean())),
        "pw_max_over_pinf": float(pw64.max() / case["wall"]["p_inf"]),
        "cf_range": [float(cf64.min()), float(cf64.max())],
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=128)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--first-cell", type=float, default=1e-3)
    ap.add_argument("--yardstick", type=float, default=1e-8,
                    help="relative perturbation of an extra FP64 run (0: skip it)")
    ap.add_argument("--save", default="", help="write the wall arrays to this .npz")
    ap.add_argument("--out", default="", help="write metrics.h5, mesh.h5 and the FP64 run's plot and "
                                              "checkpoint files (the reference's HDF5 layouts) here")
    a = ap.parse_args(argv)
    case = cases.compression_ramp(a.nx, a.ny, a.nz, first_cell=a.first_cell)
    if a.out:
        os.makedirs(a.out, exist_ok=True)
    Q64, t64 = run(case, 0, a.steps, out_dir=a.out or None)
    Q32, t32 = run(case, PREC_MIXED, a.steps)
    Qpt = run(case, 0, a.steps, perturb=a.yardstick)[0] if a.yardstick > 0 else None
    cells = a.nx * a.ny * a.nz
    out = {"case": case["name"], "steps": a.steps, "dt": case["dt"], "first_cell": a.first_cell,
           "fp64": {"ms_per_step": t64, "mcell_rhs_per_s": 3 * cells / (t64 * 1e3)},
           "mixed": {"ms_per_step": t32, "mcell_rhs_per_s": 3 * cells / (t32 * 1e3)},
           "speedup": t64 / t32, "mixed_vs_fp64": deviations(Q64, Q32, case)}
    if Qpt is not None:
        out["fp64_perturbed_vs_fp64"] = dict(deviations(Q64, Qpt, case), perturbation=a.yardstick)
    if a.save:
        w = case["wall"]
        np.savez_compressed(a.save, pw64=wall_pressure(Q64), pw32=wall_pressure(Q32),
                            cf64=skin_friction(Q64, case["x"], case["y"], w),
                            cf32=skin_friction(Q32, case["x"], case["y"], w),
                            **({} if Qpt is None else dict(pwpt=wall_pressure(Qpt),
                                                         cfpt=skin_friction(Qpt, case["x"], case["y"], w))))
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)

"""Profiling driver: set up a workload and run a few RHS evaluations through the C ABI.

Used under ncu to capture the kernels of one RHS with few launches before them:

  python -m flame3d_mhd_gb300.profile --case sod --nx 256 --ny 64 --nz 64 --reps 2
  ncu --set full --clock-control none -k regex:k_sweep -s 3 -c 3 -o prof \
      python -m flame3d_mhd_gb300.profile --case sod --reps 2

The first RHS evaluation is a warm-up (its launches are the ones skipped with -s).
With --adjoint the workload is the viscous curvilinear Taylor-Green vortex (--nx cells per
side, FP64, component-wise) and each repetition is one RK3 step VJP (f3d_rk3_step_vjp).
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np
import torch

from . import cases
from .abi import PREC_REF32
from .cases import params_copy
from .solver import Flame3D


def setup(case: str, nx: int, ny: int, nz: int, character: int = 1, precision: int = 0, scheme: int = 0):
    if case == "sod":
        c = cases.sod(nx, ny, nz, character=character)
    elif case == "tgv_viscous":
        c = cases.tgv_viscous_curvilinear(nx)
    elif case == "tgv":
        c = cases.tgv(nx, character=character)
    else:
        raise ValueError(case)
    P = c["params"]
    P.precision = precision
    P.scheme = scheme
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    if precision == PREC_REF32:
        # the reference's Float32 arrays: metrics computed in FP64 by an FP64 context, then
        # Float32 copies of them and of the state (as the reference reads metrics.h5)
        g = Flame3D(params_copy(P, precision=0))
        ms, J = g.compute_metrics(dev(c["x"]), dev(c["y"]), dev(c["z"]))
        g.close()
        s = Flame3D(P)
        s.set_metrics([m.float() for m in ms], J.float())
        Q = dev(c["Q"]).float()
        U = s.field(5)
        s.prim2c(U, Q)
        s.fillGhost(Q, U)
        return s, c, U, Q
    s = Flame3D(P)
    ms, J = s.compute_metrics(dev(c["x"]), dev(c["y"]), dev(c["z"]))
    s.set_metrics(ms, J)
    xyz = [dev(c[k]) for k in ("x", "y", "z")]
    s.set_coordinates(*xyz)
    Q = dev(c["Q"])
    U = s.field(5)
    s.prim2c(U, Q)
    s.fillGhost(Q, U)
    return s, c, U, Q


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default=None, choices=["sod", "tgv", "tgv_viscous"],
                    help="default: sod, or tgv_viscous with --adjoint")
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--nz", type=int, default=64)
    ap.add_argument("--character", type=int, default=1)
    ap.add_argument("--precision", type=int, default=0, help="0 FP64, 1 mixed, 2 the reference's Float32 form")
    ap.add_argument("--scheme", type=int, default=0, help="0 FDM, 1 FVM eigen, 2 FVM component-wise")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--step", action="store_true", help="profile_step instead of rhs (per-kernel event times)")
    ap.add_argument("--adjoint", action="store_true", help="RK3 step VJPs")
    a = ap.parse_args(argv)
    if a.case is None:
        a.case = "tgv_viscous" if a.adjoint else "sod"
    s, c, U, Q = setup(a.case, a.nx, a.ny, a.nz, a.character, a.precision, a.scheme)
    out = s.field(5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.reps):
        if a.adjoint:
            s.rk3_step_vjp(c["dt"], U, torch.ones_like(U), out)
        elif a.step:
            Un = s.field(5)
            print(json.dumps(s.profile_step(U, Un, Q, c["dt"])))
        else:
            s.rhs(Q, out)
    torch.cuda.synchronize()
    print(json.dumps({"case": a.case, "n": [a.nx, a.ny, a.nz], "reps": a.reps,
                      "ms_per_rep": (time.perf_counter() - t0) / a.reps * 1e3}), file=sys.stderr)
    s.close()


if __name__ == "__main__":
    main()

"""The reference's driver on one GPU: run.jl's configuration and solver.jl's `time_step`
(:191-509) around the library, with the reference's files in and out.

  python -m flame3d_mhd_gb300.run --mesh mesh.h5 --metrics metrics.h5 --out DIR [options]

Set-up as solver.jl:191-343: the grid dimensions and coordinates from mesh.h5 (ghosts by the
solver's extrapolation), the nine metrics and J from metrics.h5, the state from a checkpoint
(`--restart CHK/chk-N.h5`, :211-216) or the uniform free stream of boundary.jl:163-193
(rho 1, u 0.5, p 1/1.4), then prim2c and the ghost fill. Main loop as :409-509: step tt runs
while tt dt <= Time and tt <= maxStep (Float32 arithmetic, as run.jl declares dt and Time),
the stages and the filter inside the library's graph-captured steps; every 10 steps a
progress line and the NaN check (exit status 1 on NaN, as MPI.Abort); plot files (with XDMF,
or the single-dataset form), checkpoints and the running average on the reference's
conditions (tt % step == 0, |Time - dt tt| < dt, tt == maxStep). Defaults are run.jl's:
viscous, finite volume with eigen (Roe-characteristic) reconstruction, SW splitting,
hybrid thresholds 0.05 / 1 / 10, dt 1e-4, plot files every 5000 steps.

The plot files' phi is the shock sensor of the written state (the reference writes the
sensor its last stage computed from that stage's input); 0 in the Float32 form.
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import sys
import time

import numpy as np
import torch

from . import files
from .abi import (FILTER_LINEAR, FILTER_NONLINEAR, LES_SMAGORINSKY, LES_WALE, PREC_FP64, PREC_MIXED, PREC_REF32,
                  SCHEME_FDM, SCHEME_FVM_CONS, SCHEME_FVM_EIGEN, make_params)
from .solver import Flame3D, side_stream

f32 = np.float32


def n_steps(dt: float, total_time: float, max_step: int) -> int:
    """The last step of solver.jl:409-412: tt = 1 .. ceil(Time / dt) while tt dt <= Time and
    tt <= maxStep, in Float32."""
    # tt dt grows with tt, so the last step is the largest tt <= min(ceil(Time / dt), maxStep)
    # with tt dt <= Time
    n = min(int(math.ceil(float(f32(total_time) / f32(dt)))), max_step)
    while n > 0 and f32(n) * f32(dt) > f32(total_time):
        n -= 1
    return max(n, 0)


def output_due(tt: int, every: int, dt: float, total_time: float, max_step: int) -> bool:
    """IO.jl's condition for a plot / checkpoint file at step tt (IO.jl:3, 116, 155)."""
    return (tt % every == 0 or abs(f32(total_time) - f32(dt) * f32(tt)) < f32(dt) or tt == max_step)


def events(tt: int, a) -> set:
    """What happens after step tt: 'print' (every 10), 'plot', 'chk', 'avg_add', 'avg_write'."""
    ev = set()
    if tt % 10 == 0:
        ev.add("print")
    if a.plt_out and output_due(tt, a.step_plt, a.dt, a.time, a.max_step):
        ev.add("plot")
    if a.chk_out and output_due(tt, a.step_chk, a.dt, a.time, a.max_step):
        ev.add("chk")
    if a.average and tt <= a.avg_step * a.avg_total:
        if tt % a.avg_step == 0:
            ev.add("avg_add")
        if tt == a.avg_step * a.avg_total:
            ev.add("avg_write")
    return ev


def parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(description="run.jl + solver.jl's time_step on one GPU")
    ap.add_argument("--mesh", default="mesh.h5")
    ap.add_argument("--metrics", default="metrics.h5")
    ap.add_argument("--out", default=".", help="where PLT/, CHK/ and AVG/ go")
    ap.add_argument("--restart", default="none", help="a checkpoint file CHK/chk-N.h5, or none")
    ap.add_argument("--restart-nprocs", type=int, nargs=3, default=[1, 1, 1], metavar=("PX", "PY", "PZ"),
                    help="the rank layout of the run that wrote the checkpoint (run.jl's Nprocs)")
    ap.add_argument("--precision", choices=["fp64", "mixed", "ref32"], default="fp64")
    ap.add_argument("--scheme", choices=["fvm-eigen", "fvm", "fdm"], default="fvm-eigen",
                    help="finite volume with eigen / component-wise reconstruction, or finite difference")
    ap.add_argument("--character", type=int, default=1)
    ap.add_argument("--split", choices=["SW", "LF", "VL", "AUSM"], default="SW")
    ap.add_argument("--inviscid", action="store_true")
    ap.add_argument("--phi", type=float, nargs=3, default=[0.05, 1.0, 10.0], metavar=("PHI1", "PHI2", "PHI3"))
    ap.add_argument("--dt", type=float, default=1e-4)
    ap.add_argument("--time", type=float, default=100.0)
    ap.add_argument("--max-step", type=int, default=200000)
    ap.add_argument("--lts", action="store_true")
    ap.add_argument("--lts-cfl", type=float, default=0.5)
    ap.add_argument("--les", choices=["none", "smag", "wale"], default="none")
    ap.add_argument("--filtering", choices=["none", "linear", "nonlinear"], default="none")
    ap.add_argument("--filtering-interval", type=int, default=100)
    ap.add_argument("--filtering-rth", type=float, default=1e-5)
    ap.add_argument("--filtering-s0", type=float, default=1.0)
    ap.add_argument("--no-plt", dest="plt_out", action="store_false")
    ap.add_argument("--plt-h5", dest="plt_xdmf", action="store_false", help="one Q dataset instead of XDMF")
    ap.add_argument("--step-plt", type=int, default=5000)
    ap.add_argument("--plt-compress-level", type=int, default=1)
    ap.add_argument("--chk-out", action="store_true")
    ap.add_argument("--step-chk", type=int, default=5000)
    ap.add_argument("--chk-compress-level", type=int, default=1)
    ap.add_argument("--average", action="store_true")
    ap.add_argument("--avg-step", type=int, default=10)
    ap.add_argument("--avg-total", type=int, default=2000)
    ap.add_argument("--avg-compress-level", type=int, default=1)
    return ap


def setup(a):
    """The context, coordinates, metrics and initial state (solver.jl:191-343)."""
    from . import h5
    with h5.H5File(a.mesh) as f:
        nx, ny, nz = (int(f[k]) for k in ("Nx", "Ny", "Nz"))
    prec = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "ref32": PREC_REF32}[a.precision]
    scheme = {"fvm-eigen": SCHEME_FVM_EIGEN, "fvm": SCHEME_FVM_CONS, "fdm": SCHEME_FDM}[a.scheme]
    P = make_params(nx, ny, nz, precision=prec, scheme=scheme, character=a.character, split=a.split,
                    viscous=0 if a.inviscid else 1, phi1=a.phi[0], phi2=a.phi[1], phi3=a.phi[2],
                    lts=int(a.lts), lts_cfl=a.lts_cfl,
                    les={"none": 0, "smag": LES_SMAGORINSKY, "wale": LES_WALE}[a.les],
                    filter={"none": 0, "linear": FILTER_LINEAR, "nonlinear": FILTER_NONLINEAR}[a.filtering],
                    filter_interval=a.filtering_interval, filter_rth=a.filtering_rth, filter_s0=a.filtering_s0)
    s = Flame3D(P)
    dtype = np.float32 if prec == PREC_REF32 else np.float64
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=dtype)).cuda()
    m, J = files.read_metrics(a.metrics, dtype=dtype)
    s.set_metrics([dev(x) for x in m], dev(J))
    if scheme != SCHEME_FDM:
        s.set_coordinates(*(dev(c) for c in files.read_mesh(a.mesh)))
    if a.restart != "none":
        Q = dev(files.assemble_checkpoint(a.restart, tuple(a.restart_nprocs)))
    else:  # boundary.jl:163-193: the free stream at interior cells, ghosts from fillGhost
        rho, u, p = dtype(1.0), dtype(0.5), dtype(1.0) / dtype(1.4)
        q = np.zeros((6,) + s.shape3, dtype)
        I = (slice(4, -4),) * 3
        q[0][I], q[1][I], q[4][I] = rho, u, p
        q[5][I] = p / (rho * dtype(P.rg))
        Q = dev(q)
    U, Un = s.field(5), s.field(5)
    s.prim2c(U, Q)
    s.fillGhost(Q, U)
    return s, P, U, Un, Q


def main(argv=None) -> int:
    a = parser().parse_args(argv)
    dt = float(f32(a.dt))  # run.jl's dt is Float32
    s, P, U, Un, Q = setup(a)
    last = n_steps(a.dt, a.time, a.max_step)
    Qavg = torch.zeros_like(Q) if a.average else None
    phi = s.field(1)
    cells = P.nx * P.ny * P.nz
    t0, tt = time.perf_counter(), 0
    with side_stream() as stream:
        while tt < last:
            nxt = tt + 1  # run to the next step with an event (graph replays in between)
            while nxt < last and not events(nxt, a):
                nxt += 1
            s.time_step(U, Un, Q, dt, nxt - tt)
            tt = nxt
            ev = events(tt, a)
            if "print" in ev:
                stream.synchronize()
                print(f"Step: {tt}\tTime: {tt * dt:.2e}\tWall time: {datetime.datetime.now().isoformat()}",
                      flush=True)
                if not s.check_finite(U):
                    print("Oops, NaN detected", flush=True)
                    s.close()
                    return 1
            if "plot" in ev:
                if a.plt_xdmf:
                    if not s.ref32:  # the Float32 form has no sensor entry: phi stays 0 there
                        s.shockSensor(phi, Q)
                    files.plotFile_xdmf(a.out, tt, Q, phi, dt, compress=a.plt_compress_level or None)
                else:
                    files.plotFile_h5(a.out, tt, Q, compress=a.plt_compress_level or None)
            if "chk" in ev:
                files.checkpointFile(a.out, tt, Q, compress=a.chk_compress_level or None)
            if "avg_add" in ev:
                Qavg += Q / a.avg_total
            if "avg_write" in ev:
                print("average done", flush=True)
                files.averageFile(a.out, tt, Qavg, compress=a.avg_compress_level or None)
        stream.synchronize()
    wall = time.perf_counter() - t0
    finite = s.check_finite(U)
    print(json.dumps({"steps": tt, "time": tt * dt, "wall_s": wall, "finite": finite,
                      "mcell_updates_per_s": cells * tt / wall / 1e6 if wall > 0 else None}))
    s.close()
    return 0 if finite else 1


if __name__ == "__main__":
    sys.exit(main())

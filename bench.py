#!/usr/bin/env python
"""Benchmark: FP64 SSP-RK3 steps of the Flame3D finite-difference RHS on one GB300.

Workload (the configuration the headline metric is quoted on): Sod shock tube on a
perturbed curvilinear grid, 256 x 64 x 64 interior cells (264 x 72 x 72 with ghosts),
x = xi + 0.02 sin(2 pi eta) sin(2 pi zeta) and cyclic, metrics and J computed from these
coordinates on the device, hybrid UP7/WENO7/WENO5/NND2 with the shock sensor,
characteristic-wise reconstruction, Steger-Warming splitting, inviscid, zero-gradient x and
periodic y, z. A step is one SSP-RK3 time step = 3 RHS evaluations; the metric counts
interior cells x RHS evaluations per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation (the C++ restatement
in oracle/, OpenMP over all host cores) on the same workload; Julia is not available to
run the reference's own code. Under torchrun each rank runs an independent replica (the
path is single-GPU by design: no sharding, no collectives); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-RHS/s FP64 vs mixed at stated L-inf err; adjoint/forward step time"
UNIT = "Mcell-RHS/s"
WORKLOAD = dict(nx=256, ny=64, nz=64)
NG = 4

# Algorithmic (compulsory) bytes per interior cell of each kernel of one stage, FP64:
# what the kernel must read and write at least once given its interface.
#   sweep (first, OUT_SET): Q 6 + c 1 + metric row 3 + A/|A| 3 + |A| 1 + phi 1 read, acc 5 write
#   sweep (second, OUT_ADD): the same reads + acc 5 read + acc 5 write
#   sweep (last, OUT_STAGE): the same reads + acc 5 + U 5 + Un 5 (stages 2,3) + J 1 read, U 5 write
#   prim_ghost_fill: U 5 read, Q 6 write;  sound_speed: T (or p, rho) read, c write;
#   shock_sensor: p read, phi write
KERNEL_BYTES_PER_CELL = {
    "sweep_xi": 8 * (15 + 5),
    "sweep_eta": 8 * (15 + 10),
    "sweep_zeta": 8 * (15 + 16 + 5),
    "prim_ghost_fill": 8 * (5 + 6),
    "sound_speed": 8 * 2,
    "shock_sensor": 8 * 2,
    "viscous_flux": 8 * (6 + 10 + 12),
}
# one RK3 step of the whole RHS: 3 x (U + 9 metrics + J read, U written) + 2 x Un read
STEP_BYTES_PER_CELL = 3 * 160 + 2 * 40

# DRAM bytes per interior cell of one launch in an RK3 stage on this workload, measured by
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none -k regex:k_sweep
#       python -m flame3d_mhd_gb300.profile --case sod --nx 256 --ny 64 --nz 64 --reps 2 --step
# (read + write bytes of each sweep divided by the interior cell count)
KERNEL_TRAFFIC_PER_CELL = {"sweep_xi": 135.2, "sweep_eta": 195.7, "sweep_zeta": 297.1}


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 50 ms while running (the FP64 timed
    region of the default run lasts about 0.3 s)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float) -> dict:
        rows = [r for t, r in self.rows if t0 <= t <= t1] or [r for _, r in self.rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x: float, device=None) -> float:
    """Maximum of x over the ranks of the default process group (x itself when there is none).
    Host-side control only: one scalar per timed run, no data-path collective."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(target_s: float = 12.0, max_steps: int = 8) -> dict:
    """The oracle (C++ restatement of the reference algorithm, OpenMP on every host core; its
    RHS and RK3 steps equal the reference's kernels translated into Python bit for bit on the
    fixture cases) on the same workload: one untimed step, then whole RK3 steps until about
    target_s."""
    import numpy as np

    from flame3d_mhd_gb300 import cases
    from oracle import oracle as orc
    threads = orc.set_threads(os.cpu_count() or 1)
    c = cases.sod(**WORKLOAD)
    P = c["params"]
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    Un = np.zeros_like(U)
    s = orc.PersistentSolver(P, m, J)
    s.rk3(1, c["dt"], U, Un, Q)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and (time.perf_counter() - t0) < target_s:
        s.rk3(1, c["dt"], U, Un, Q)
        steps += 1
    dt = time.perf_counter() - t0
    s.close()
    cells = WORKLOAD["nx"] * WORKLOAD["ny"] * WORKLOAD["nz"]
    return {"value": cells * 3 * steps / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} SSP-RK3 steps ({3 * steps} RHS) of the {WORKLOAD['nx']}x{WORKLOAD['ny']}x"
                      f"{WORKLOAD['nz']} workload after 1 untimed step, {dt:.1f} s"}


def workload_flops_per_cell() -> float:
    """Floating-point operations of one RHS per interior cell on the workload, counted
    exactly by the oracle's counting number type (add + mul + div + sqrt, an FMA counting
    as two), with this workload's own branch mix."""
    from flame3d_mhd_gb300 import cases
    from oracle import oracle as orc
    c = cases.sod(**WORKLOAD)
    P = c["params"]
    m, J, Q, _ = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    oc = orc.rhs_opcount(P, Q, m, J)
    cells = WORKLOAD["nx"] * WORKLOAD["ny"] * WORKLOAD["nz"]
    return float(oc["add"] + oc["mul"] + oc["div"] + oc["sqrt"]) / cells


def rhs_parity(rhs_gpu) -> dict:
    """The FP64 RHS of the workload's initial state against the oracle (the checker, outside
    the timed region): relative L-inf per variable, and the difference relative to the flux
    scale (per variable, max of J times the summed face fluxes the RHS differences), beside
    the oracle's own distance from an extended-precision evaluation."""
    import numpy as np

    from flame3d_mhd_gb300 import cases
    from oracle import oracle as orc
    c = cases.sod(**WORKLOAD)
    P = c["params"]
    m, J, Q, _ = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    ro = orc.rhs(P, Q, m, J)
    rl, scale = orc.rhs_ld(P, Q, m, J)
    I = (slice(NG, -NG),) * 3
    r = np.asarray(rhs_gpu)

    def rel(a, b):
        return max(float(np.abs(a[n][I] - b[n][I]).max() / np.abs(b[n][I]).max()) for n in range(5))
    scaled = max(float(np.abs(r[n][I] - ro[n][I]).max() / scale[n]) for n in range(5))
    scaled_ld = max(float(np.abs(r[n][I] - rl[n][I]).max() / scale[n]) for n in range(5))
    orc_scaled_ld = max(float(np.abs(ro[n][I] - rl[n][I]).max() / scale[n]) for n in range(5))
    return {"rhs_rel_linf": rel(r, ro), "rhs_flux_scaled": scaled, "rhs_flux_scaled_vs_extended": scaled_ld,
            "oracle_flux_scaled_vs_extended": orc_scaled_ld, "rhs_rel_linf_vs_extended": rel(r, rl),
            "oracle_rel_linf_vs_extended": rel(ro, rl), "tolerance": 1e-12,
            "note": "FP64 RHS of the initial state; flux-scaled = |a - b| / max J sum|F| per variable; "
                    "'extended' = the oracle's long-double evaluation of the reference's formulas"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    from flame3d_mhd_gb300 import cases
    from oracle import oracle as orc
    threads = orc.set_threads(os.cpu_count() or 1)
    c = cases.sod(**WORKLOAD)
    P = c["params"]
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    Un = np.zeros_like(U)
    s = orc.PersistentSolver(P, m, J)
    s.rk3(max(args.warmup, 1), c["dt"], U, Un, Q)
    t0 = time.perf_counter()
    s.rk3(args.steps, c["dt"], U, Un, Q)
    dt = time.perf_counter() - t0
    s.close()
    cells = WORKLOAD["nx"] * WORKLOAD["ny"] * WORKLOAD["nz"]
    value = cells * 3 * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sod_curvilinear_256x64x64_hybrid_char_SW_inviscid", **WORKLOAD,
                   "parallelism": "openmp", "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} SSP-RK3 steps of the full workload after {max(args.warmup, 1)} "
                                   f"untimed; C++ restatement of the reference formulas (Julia absent), equal bit "
                                   f"for bit to the reference's kernels translated into Python on the fixture cases"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ramp_leg(nx: int, ny: int, nz: int, steps: int) -> dict:
    """The viscous Mach 2.9 compression ramp (24 degrees, body-fitted grid, isothermal wall,
    1/7-power inflow, Re 1e5, Sutherland, Pr 0.72) in FP64 and in mixed precision from the
    same initial state: Mcell-RHS/s of each (CUDA events over steps - 1 graph-replayed RK3
    steps after one) and the mixed form's deviation from FP64 in wall pressure and skin
    friction after `steps` steps (max and mean, relative to the FP64 values' maximum / mean)."""
    from flame3d_mhd_gb300 import cases, ramp
    from flame3d_mhd_gb300.abi import PREC_MIXED
    case = cases.compression_ramp(nx, ny, nz)
    Q64, t64 = ramp.run(case, 0, steps, wall_only=True)
    Q32, t32 = ramp.run(case, PREC_MIXED, steps, wall_only=True)
    cells = nx * ny * nz
    return {"workload": f"{case['name']}: viscous Mach 2.9 compression ramp, 24 deg, isothermal wall, "
                        f"tanh wall-normal stretching, first cell 1e-3 delta", "steps": steps,
            "timed_steps": steps - 1,
            "fp64": {"value": 3 * cells / (t64 * 1e3), "unit": UNIT, "ms_per_step": t64},
            "mixed": {"value": 3 * cells / (t32 * 1e3), "unit": UNIT, "ms_per_step": t32},
            "speedup_mixed_vs_fp64": t64 / t32, "mixed_vs_fp64": ramp.deviations(Q64, Q32, case)}


def adjoint_cost(args, n: int = 128, steps: int = 4, workload: str = "tgv") -> dict:
    """Adjoint / forward cost of one SSP-RK3 step: the adjoint step recomputes two stage states
    and applies three RHS VJPs (f3d_rk3_step_vjp). workload "tgv": the viscous curvilinear
    Taylor-Green vortex of the adjoint configuration (n^3, Re 1600, Mach 0.1, FP64,
    component-wise hybrid; its faces all take UP7); "sod": the bench workload (shock tube
    256x64x64, characteristic-wise hybrid, inviscid), whose WENO faces exercise the
    characteristic reverse."""
    import numpy as np
    import torch

    from flame3d_mhd_gb300 import cases
    from flame3d_mhd_gb300.solver import Flame3D, side_stream
    c = cases.tgv_viscous_curvilinear(n) if workload == "tgv" else cases.sod(**WORKLOAD)
    P = c["params"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s = Flame3D(P)
    ms, J = s.compute_metrics(dev(c["x"]), dev(c["y"]), dev(c["z"]))
    s.set_metrics(ms, J)
    Q = dev(c["Q"])
    U, Un = s.field(5), s.field(5)
    s.prim2c(U, Q)
    s.fillGhost(Q, U)
    dt = c["dt"]
    Ub, Ub2 = torch.ones_like(U), s.field(5)
    with side_stream() as stream:
        s.time_step(U, Un, Q, dt, 2)
        s.rk3_step_vjp(dt, U, Ub, Ub2)
        stream.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        s.time_step(U, Un, Q, dt, steps)
        e[1].record(stream)
        e[2].record(stream)
        for _ in range(steps):
            s.rk3_step_vjp(dt, U, Ub, Ub2)
        e[3].record(stream)
        e[3].synchronize()
    fwd = e[0].elapsed_time(e[1]) / steps
    adj = e[2].elapsed_time(e[3]) / steps
    s.close()
    desc = (f"tgv{n}^3 viscous, curvilinear amp 0.05, Re 1600, Mach 0.1, FP64, component-wise hybrid"
            if workload == "tgv" else "sod_curvilinear_256x64x64, FP64, characteristic-wise hybrid, inviscid")
    cells = P.nx * P.ny * P.nz
    return {"workload": desc,
            "forward_ms_per_step": fwd, "adjoint_ms_per_step": adj, "adjoint_over_forward": adj / fwd,
            "forward_mcell_rhs_per_s": cells * 3 / (fwd / 1e3) / 1e6,
            "adjoint_includes": "recompute of 2 stage states + 3 RHS VJPs per step"}


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from flame3d_mhd_gb300 import build as fbuild
    fbuild.build()
    from flame3d_mhd_gb300 import cases
    from flame3d_mhd_gb300.solver import Flame3D, side_stream

    c = cases.sod(**WORKLOAD)
    P = c["params"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s = Flame3D(P)
    ms, J = s.compute_metrics(dev(c["x"]), dev(c["y"]), dev(c["z"]))
    s.set_metrics(ms, J)
    Q = dev(c["Q"])
    U, Un = s.field(5), s.field(5)
    s.prim2c(U, Q)
    s.fillGhost(Q, U)
    Q0, U0 = Q.clone(), U.clone()
    dt = c["dt"]
    cells = P.nx * P.ny * P.nz

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    stream = torch.cuda.Stream()

    def timed_steps(solver, U, Un, Q, steps, warmup):
        """warmup untimed steps, then `steps` timed ones (CUDA events on `stream`, barriers
        and device syncs on both sides); returns (ms, wall t0, wall t1)."""
        with side_stream(stream):
            for _ in range(warmup):
                solver.time_step(U, Un, Q, dt, 1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream.synchronize()
            barrier()
            torch.cuda.synchronize()
            t0 = time.time()
            e0.record(stream)
            solver.time_step(U, Un, Q, dt, steps)
            e1.record(stream)
            e1.synchronize()
            torch.cuda.synchronize()
            barrier()
            t1 = time.time()
        return reduce_max(e0.elapsed_time(e1), device="cuda"), t0, t1

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    ms_total, tw0, tw1 = timed_steps(s, U, Un, Q, args.steps, args.warmup)
    sampler.stop()
    U_fp64 = U.clone()
    ms_step = ms_total / args.steps
    value = ws * cells * 3 * args.steps / (ms_total / 1e3) / 1e6
    ok = s.check_finite(U)

    # mixed precision on the same workload, from the same initial state, same step count
    from flame3d_mhd_gb300.abi import PREC_MIXED
    from flame3d_mhd_gb300.cases import params_copy
    sm = Flame3D(params_copy(P, precision=PREC_MIXED))
    sm.set_metrics(ms, J)
    Um, Unm, Qm = U0.clone(), torch.zeros_like(U0), Q0.clone()
    ms_mixed, _, _ = timed_steps(sm, Um, Unm, Qm, args.steps, args.warmup)
    value_mixed = ws * cells * 3 * args.steps / (ms_mixed / 1e3) / 1e6
    Iin = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    state_err = float((Um[Iin] - U_fp64[Iin]).abs().max() / U_fp64[Iin].abs().max())

    def kinetic(Uv):
        r = Uv[Iin][0]
        return float(((0.5 * (Uv[Iin][1] ** 2 + Uv[Iin][2] ** 2 + Uv[Iin][3] ** 2) / r) / J[Iin[1:]]).sum())
    ke64, ke32 = kinetic(U_fp64), kinetic(Um)
    r64, r32 = s.rhs(Q0), sm.rhs(Q0)
    rhs_err = max(float((r32[n][Iin[1:]] - r64[n][Iin[1:]]).abs().max() / r64[n][Iin[1:]].abs().max())
                  for n in range(5))
    prof_m = {}
    with side_stream(stream):
        for _ in range(3):
            for k, (t_ms, n) in sm.profile_step(Um, Unm, Qm, dt).items():
                a = prof_m.setdefault(k, [0.0, 0])
                a[0] += t_ms
                a[1] += n
    tot_m = sum(t for t, _ in prof_m.values())
    mixed = {"value": value_mixed, "unit": UNIT, "ms_per_step": ms_mixed / args.steps,
             "speedup_vs_fp64": value_mixed / value,
             "err_vs_fp64": {"rhs_rel_linf_initial_state": rhs_err,
                             "state_rel_linf_after_steps": state_err,
                             "kinetic_energy_rel": abs(ke32 - ke64) / abs(ke64) if ke64 else None,
                             "steps": args.steps + args.warmup},
             "shares": {k: round(v[0] / tot_m, 4) for k, v in sorted(prof_m.items())},
             "step_hbm_frac": STEP_BYTES_PER_CELL * cells / (ms_mixed / args.steps / 1e3) / 1e9 / load_peaks()["hbm_gbs"]}
    sm.close()

    # the reference's own Float32 arrays and arithmetic (F3D_PREC_REF32), same workload and
    # step count, from the Float32 copy of the same initial state
    from flame3d_mhd_gb300.abi import PREC_REF32
    sr = Flame3D(params_copy(P, precision=PREC_REF32))
    sr.set_metrics([a.float() for a in ms], J.float())
    Ur, Unr, Qr = U0.float(), torch.zeros_like(U0, dtype=torch.float32), Q0.float()
    sr.q_from_u(Ur, Qr)
    ms_r32, _, _ = timed_steps(sr, Ur, Unr, Qr, args.steps, args.warmup)
    ref32 = {"value": ws * cells * 3 * args.steps / (ms_r32 / 1e3) / 1e6, "unit": UNIT,
             "ms_per_step": ms_r32 / args.steps,
             "form": "the reference's Float32 arrays and arithmetic (WENO7 weights in FP64)",
             "state_rel_linf_vs_fp64_after_steps":
                 float((Ur[Iin].double() - U_fp64[Iin]).abs().max() / U_fp64[Iin].abs().max()),
             "state_finite": bool(torch.isfinite(Ur).all())}
    sr.close()

    # the reference's default scheme (run.jl:64-65: finite volume, eigen reconstruction,
    # HLLC) on the same workload and step count, FP64
    from flame3d_mhd_gb300.abi import SCHEME_FVM_EIGEN
    sf = Flame3D(params_copy(P, scheme=SCHEME_FVM_EIGEN))
    sf.set_metrics(ms, J)
    sf.set_coordinates(dev(c["x"]), dev(c["y"]), dev(c["z"]))
    Uf, Unf, Qf = U0.clone(), torch.zeros_like(U0), Q0.clone()
    ms_fvm, _, _ = timed_steps(sf, Uf, Unf, Qf, args.steps, args.warmup)
    fvm = {"value": ws * cells * 3 * args.steps / (ms_fvm / 1e3) / 1e6, "unit": UNIT,
           "ms_per_step": ms_fvm / args.steps, "scheme": "finite volume, Roe-characteristic WENO7/WENO5/minmod "
           "of U + HLLC (FVM.jl)", "state_finite": bool(sf.check_finite(Uf))}
    sf.close()
    adjoint = adjoint_cost(args)
    adjoint["characteristic"] = adjoint_cost(args, workload="sod")
    # the configurations the metric is quoted on: the compression ramp at 512x256x128 and at
    # 1024x384x192, FP64 and mixed precision from the same state
    ramps = {} if args.no_ramp else {"config3_ramp_512x256x128": ramp_leg(512, 256, 128, 30),
                                     "config5_ramp_1024x384x192": ramp_leg(1024, 384, 192, 10)}

    # per-kernel device times of single steps (events between launches, outside the timed loop)
    prof = {}
    with side_stream(stream):
        for _ in range(3):
            for k, (t_ms, n) in s.profile_step(U, Un, Q, dt).items():
                a = prof.setdefault(k, [0.0, 0])
                a[0] += t_ms
                a[1] += n
    launches_per_step = sum(n for _, n in prof.values()) // 3
    total_ms = sum(t for t, _ in prof.values())
    top = max(prof, key=lambda k: prof[k][0])
    top_avg_ms = prof[top][0] / prof[top][1]
    peaks = load_peaks()
    alg = KERNEL_BYTES_PER_CELL[top] * cells
    achieved = alg / (top_avg_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": KERNEL_TRAFFIC_PER_CELL[top] * cells if top in KERNEL_TRAFFIC_PER_CELL else None,
                "traffic_source": "ncu DRAM bytes per cell of the stage-mode sweep on this workload", "kernel": top,
                "peak_source": peaks["source"],
                "alg_bytes_per_launch": alg, "avg_launch_ms": top_avg_ms,
                "shares": {k: round(v[0] / total_ms, 4) for k, v in sorted(prof.items())}}
    step_gbs = STEP_BYTES_PER_CELL * cells / (ms_step / 1e3) / 1e9

    # end to end through the public API with host buffers, per step: H2D of the conserved
    # state U from pinned memory, its primitive state and ghost layers on the device
    # (f3d_c2prim + f3d_fill_ghosts), one step, D2H of U. Two contexts with their own state
    # arrays alternate, so the copies of one step (on an H2D and a D2H stream, one copy
    # engine each way) overlap the other's compute.
    U_h = U0.cpu().pin_memory()
    outs = [torch.empty_like(U_h).pin_memory() for _ in range(2)]
    s2 = Flame3D(P)
    s2.set_metrics(ms, J)
    ctxs = [s, s2]
    bufs = [(U, Un, Q), (torch.empty_like(U), torch.empty_like(Un), torch.empty_like(Q))]
    h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    ev_free = [torch.cuda.Event() for _ in range(2)]
    e2e_steps = max(4, min(args.steps, 20))

    def e2e_loop(nsteps):
        h2d.wait_stream(stream)
        for it in range(nsteps):
            k = it % 2
            Uk, Unk, Qk = bufs[k]
            with torch.cuda.stream(h2d):
                if it >= 2:
                    h2d.wait_event(ev_free[k])  # the buffer's previous result has left
                Uk.copy_(U_h, non_blocking=True)
                ev_in[k].record(h2d)
            stream.wait_event(ev_in[k])
            with torch.cuda.stream(stream):
                ctxs[k].q_from_u(Uk, Qk)
                ctxs[k].time_step(Uk, Unk, Qk, dt, 1)
                ev_done[k].record(stream)
            d2h.wait_event(ev_done[k])
            with torch.cuda.stream(d2h):
                outs[k].copy_(Uk, non_blocking=True)
                ev_free[k].record(d2h)
        stream.wait_stream(d2h)

    with side_stream(stream):
        e2e_loop(2)  # capture both contexts' step graphs
        stream.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        e2e_loop(e2e_steps)
        f1.record(stream)
        f1.synchronize()
    e2e_ms = f0.elapsed_time(f1) / e2e_steps
    e2e_value = ws * cells * 3 / (e2e_ms / 1e3) / 1e6
    nbytes = U.numel() * 8
    e2e_ok = bool(torch.equal(outs[(e2e_steps - 1) % 2], outs[(e2e_steps - 2) % 2]))  # same input, same result
    s2.close()

    clocks = sampler.summary(tw0, tw1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "sod_curvilinear_256x64x64_hybrid_char_SW_inviscid", **WORKLOAD,
                   "precision": "fp64", "step": "one SSP-RK3 step (3 RHS)", "parallelism": f"replicas{ws}",
                   "l2": "inputs larger than L2 (state + metrics + scratch ~0.5 GB)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "steps": e2e_steps, "results_agree": e2e_ok,
                "per_step": "H2D of U from pinned host memory, Q and ghosts from it on the device, one RK3 "
                            "step, D2H of U; two contexts alternate so one step's copies overlap the other's "
                            "compute"},
        # one time_step call: the sound speed of Q once, then per step the three stages, whose
        # primitive fills rewrite it (profile_step's count includes stage 1's sound speed)
        "gpu_launches": (launches_per_step - 1) * args.steps + 1,
        "roofline": roofline,
        "roofline_step": {"bound": "hbm", "achieved": step_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                          "frac": step_gbs / peaks["hbm_gbs"], "alg_bytes_per_cell_step": STEP_BYTES_PER_CELL},
        "mcell_updates_per_s": value / 3,
        "mixed": mixed,
        "ref32": ref32,
        "fvm": fvm,
        "adjoint": adjoint,
        **ramps,
        "clocks": clocks,
        "state_finite": bool(ok),
    }
    # the FP64 form's binding roof is the FP64 pipe: achieved flop rate of the whole RHS
    # against the FMA-chain peak measured on this GPU now
    from flame3d_mhd_gb300.solver import measure_pipes
    fp64_peak, fp32_peak = measure_pipes()
    line["roofline_fp64_pipe"] = {"bound": "fp64", "peak": fp64_peak, "unit": "TFLOP/s", "fp32_peak": fp32_peak,
                                  "achieved": None, "frac": None, "flops_per_cell_rhs": None,
                                  "note": "flops from the oracle's exact op count (CPU leg); GPU divides "
                                          "and square roots cost ~10 FMA slots each but count as 1"}
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["parity"] = rhs_parity(r64.cpu().numpy())
        line["cpu_baseline"] = cpu_sample()
        f = workload_flops_per_cell()
        ach = f * value * 1e6 / ws / 1e12
        line["roofline_fp64_pipe"].update(achieved=ach, frac=ach / fp64_peak, flops_per_cell_rhs=f)
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-ramp", action="store_true", help="skip the compression-ramp legs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

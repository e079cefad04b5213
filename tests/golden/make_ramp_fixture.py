"""Make tests/golden/swept_ramp_ref.npz from the reference's own grid generator.

The reference's SCU-benchmark/swept-compression-ramp.c is compiled unmodified by
`make -C oracle ref REF=<reference tree>` (against the MPI stand-in oracle/ref_ramp/mpi.h)
at gcc's default optimisation level and at -O2; this script runs both builds and stores
  - the coordinates of three small grids (one process; two processes with a 30-degree sweep;
    three processes with 7 planes and an 18-degree ramp), from the default build;
  - SHA-256 digests of the coordinates of the benchmark grid of its
    swept-compression-grid.in (1000 x 240 x 100) from both builds, which differ in the last
    bit of one point per plane (gcc -O2 squares pow(v, 2) by multiplication).

    python tests/golden/make_ramp_fixture.py --ref <reference tree>
"""
from __future__ import annotations

import argparse
import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

SMALL = dict(nx=64, ny=24, nz=6, nprocs=1, nx_inlet=40, nx_corner=20, nx_buff=4, dx_inlet=0.9, lx_inlet=30.0,
             lx_corner=8.0, alfax_buff=1.05, sw_angle=0.0, comp_angle=24.0, high=6.0, hy_wall=0.01, lz=3.0)
VARIANTS = {"one_process": {}, "two_processes_swept": dict(sw_angle=30.0, nprocs=2),
            "three_processes": dict(nprocs=3, nz=7, comp_angle=18.0)}
BENCHMARK = dict(nx=1000, ny=240, nz=100, nprocs=1, nx_inlet=680, nx_corner=300, nx_buff=20, dx_inlet=0.5,
                 lx_inlet=300.0, lx_corner=50.0, alfax_buff=1.05, sw_angle=0.0, comp_angle=24.0, high=35.0,
                 hy_wall=0.01, lz=14.0)


def digest(x, y, z) -> str:
    h = hashlib.sha256()
    for a in (x, y, z):
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference source tree")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={args.ref}"], check=True)
    from oracle.ref_ramp import run_ref
    out = {}
    meta = {"small": SMALL, "variants": VARIANTS, "benchmark": BENCHMARK}
    for name, kw in VARIANTS.items():
        q = dict(SMALL, **kw)
        x, y, z = run_ref.run(q)
        out[f"{name}_x"], out[f"{name}_y"], out[f"{name}_z"] = x, y, z
    meta["benchmark_sha256_O0"] = digest(*run_ref.run(BENCHMARK))
    meta["benchmark_sha256_O2"] = digest(*run_ref.run(BENCHMARK, o2=True))
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(HERE / "swept_ramp_ref.npz", **out)
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()

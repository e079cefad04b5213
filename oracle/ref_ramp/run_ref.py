"""Run the reference's own grid generator (SCU-benchmark/swept-compression-ramp.c, compiled
unmodified into oracle/_ref/ by `make -C oracle ref` against the MPI stand-in of
oracle/ref_ramp/mpi.h) and read back the OCFD3d-Mesh.dat it writes.

TEST INFRASTRUCTURE ONLY: used by tests/ and tests/golden/make_ramp_fixture.py to pin the
restated generator of flame3d_mhd_gb300/meshgen.py on the program itself.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BIN = HERE.parent / "_ref" / "swept_compression_ramp"        # gcc's default optimisation level
BIN_O2 = HERE.parent / "_ref" / "swept_compression_ramp_O2"  # -O2: pow(v, 2) becomes v * v

# the parameter file's six title / value line pairs (Read_parameter, swept-compression-ramp.c:78-105)
_FIELDS = (("nx", "ny", "nz", "nprocs"), ("nx_inlet", "nx_corner", "nx_buff"),
           ("dx_inlet", "lx_inlet", "lx_corner", "alfax_buff"), ("sw_angle", "comp_angle"),
           ("high", "hy_wall", "lz"), ("tec1", "mesh2d", "tec2"))


def available() -> bool:
    if not (BIN.exists() and BIN_O2.exists()):
        subprocess.run(["make", "-s", "-C", str(HERE.parent), "ref"], check=False, capture_output=True)
    return BIN.exists() and BIN_O2.exists()


def write_params(path: Path, p: dict) -> None:
    q = dict(tec1=0, mesh2d=0, tec2=0)
    q.update(p)
    lines = []
    for names in _FIELDS:
        lines.append("  ".join(names))
        lines.append("  ".join(repr(q[n]) if isinstance(q[n], float) else str(int(q[n])) for n in names))
    path.write_text("\n".join(lines) + "\n")


def run(p: dict, o2: bool = False) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Coordinates (Nz, Ny, Nx) of the program's OCFD3d-Mesh.dat for parameters p (the keys of
    meshgen.SWEPT_DEFAULTS, all given). Its p["nprocs"] ranks run one after another. o2: the
    -O2 build."""
    if not available():
        raise FileNotFoundError(f"{BIN} is not built (the reference source is absent)")
    nx, ny, nz, nproc = (int(p[k]) for k in ("nx", "ny", "nz", "nprocs"))
    with tempfile.TemporaryDirectory() as d:
        write_params(Path(d) / "swept-compression-grid.in", p)
        for r in range(nproc):
            env = dict(os.environ, F3D_MPI_RANK=str(r), F3D_MPI_SIZE=str(nproc))
            subprocess.run([str(BIN_O2 if o2 else BIN)], cwd=d, env=env, check=True, capture_output=True)
        rec = nx * ny * 8
        raw = np.fromfile(Path(d) / "OCFD3d-Mesh.dat", dtype=np.uint8)
        if raw.size != 3 * nz * (rec + 8):
            raise ValueError(f"OCFD3d-Mesh.dat has {raw.size} bytes for {nx}x{ny}x{nz}")
        recs = raw.reshape(3, nz, rec + 8)
        data = recs[:, :, 4:rec + 4].copy().view("<f8").reshape(3, nz, ny, nx)
        return data[0].copy(), data[1].copy(), data[2].copy()

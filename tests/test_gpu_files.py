"""The reference's HDF5 files from a GPU run: the ramp driver's --out writes metrics.h5,
mesh.h5, the plot (+ XDMF) and checkpoint files; their contents are the device metrics and
the final state rounded to Float32, and a restart from the checkpoint file is bitwise the
restart from the same Float32 state held in memory."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest
import torch

from flame3d_mhd_gb300 import cases, files, h5, ramp
from flame3d_mhd_gb300.solver import Flame3D, side_stream

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(NG, -NG),) * 3


def test_ramp_run_writes_the_reference_files(gpu_lib, tmp_path):
    nx, ny, nz, steps = 32, 24, 4, 3
    out = str(tmp_path)
    ramp.main(["--nx", str(nx), "--ny", str(ny), "--nz", str(nz), "--steps", str(steps), "--first-cell", "1e-2",
               "--yardstick", "0", "--out", out])
    case = cases.compression_ramp(nx, ny, nz, first_cell=1e-2)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s = Flame3D(case["params"])
    ms, J = s.compute_metrics(to(case["x"]), to(case["y"]), to(case["z"]))
    # metrics.h5: the device metrics in Float32, ghosts included
    mf, Jf = files.read_metrics(os.path.join(out, "metrics.h5"))
    for a, b in zip(mf + [Jf], ms + [J]):
        assert np.array_equal(a, b.cpu().numpy().astype(np.float32).astype(np.float64))
    # mesh.h5: the interior coordinates; read back with the solver's ghost extrapolation
    X, Y, Z = files.read_mesh(os.path.join(out, "mesh.h5"))
    for A, a in zip((X, Y, Z), (case["x"], case["y"], case["z"])):
        assert A.shape == a.shape and np.array_equal(A[I], a[I].astype(np.float32))
    # plot file and XDMF; the checkpoint holds the same state with ghosts
    Qc = files.read_checkpoint(os.path.join(out, "CHK", f"chk-{steps}.h5"))
    plt = h5.read(os.path.join(out, "PLT", f"plt-{steps}.h5"))
    for n, name in enumerate(files.PRIM_NAMES):
        assert np.array_equal(plt[name], Qc[n][I])
    assert np.isfinite(plt["phi"]).all() and plt["phi"].shape == (nz, ny, nx)
    assert np.isfinite(Qc).all() and (Qc[0] > 0).all()
    ET.parse(os.path.join(out, "PLT", f"plt-{steps}.xmf"))

    # restart from the checkpoint file = restart from the same Float32 state in memory
    def restart(Q32):
        s.set_metrics(ms, J)
        s.set_inflow_profile(0, to(case["profile"]))
        Q = to(Q32.astype(np.float64))
        U, Un = s.field(5), s.field(5)
        s.prim2c(U, Q)
        s.fillGhost(Q, U)
        with side_stream():
            s.time_step(U, Un, Q, case["dt"], 2)
        torch.cuda.synchronize()
        return U.cpu().numpy()

    U_file = restart(Qc)
    # the same final state from memory: c2Prim of the final U, rounded to Float32
    s2 = Flame3D(case["params"])
    s2.set_metrics(ms, J)
    s2.set_inflow_profile(0, to(case["profile"]))
    Q0 = to(case["Q"])
    U, Un = s2.field(5), s2.field(5)
    s2.prim2c(U, Q0)
    s2.fillGhost(Q0, U)
    with side_stream():
        s2.time_step(U, Un, Q0, case["dt"], steps)
    Qf = s2.q_from_u(U).cpu().numpy().astype(np.float32)
    s2.close()
    assert np.array_equal(Qf, Qc)
    assert np.array_equal(U_file, restart(Qf))
    s.close()

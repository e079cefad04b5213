"""The run.jl / solver.jl driver: loop bounds and output conditions in Float32 (CPU), and an
end-to-end run from the reference's files with plot, checkpoint and average output and a
restart (GPU)."""
import os

import numpy as np
import pytest

from flame3d_mhd_gb300 import files, h5, meshgen, run


def test_loop_bounds_and_output_conditions():
    # Float32 arithmetic of solver.jl:409-412 and IO.jl's conditions
    assert run.n_steps(1e-4, 100.0, 200000) == 200000
    assert run.n_steps(1e-4, 100.0, 10 ** 7) == 1000000
    assert run.n_steps(1e-3, 0.025, 100) == 25
    assert run.n_steps(0.1, 1.0, 100) == 10
    assert run.n_steps(0.3, 0.2, 100) == 0
    brute = lambda dt, T, m: max([0] + [t for t in range(1, int(np.ceil(np.float32(T) / np.float32(dt))) + 1)
                                        if np.float32(t) * np.float32(dt) <= np.float32(T) and t <= m])
    for dt, T, m in ((1e-3, 0.025, 100), (7e-3, 0.1, 100), (0.01, 0.05, 3), (1e-4, 0.0123, 1000)):
        assert run.n_steps(dt, T, m) == brute(dt, T, m)
    a = run.parser().parse_args(["--step-plt", "10", "--chk-out", "--step-chk", "20", "--average", "--avg-step", "5",
                                 "--avg-total", "2", "--dt", "1e-3", "--time", "0.025", "--max-step", "100"])
    assert run.events(10, a) == {"print", "plot", "avg_add", "avg_write"}
    assert run.events(20, a) == {"print", "plot", "chk"}
    assert run.events(5, a) == {"avg_add"}
    assert "plot" in run.events(25, a) and "chk" in run.events(25, a)  # |Time - dt tt| < dt
    assert run.events(7, a) == set()


@pytest.mark.gpu
def test_run_from_the_reference_files(gpu_lib, tmp_path):
    X, Y, Z = meshgen.flat_plate_grid(24, 20, 8)
    meshgen.reference_files(str(tmp_path), X, Y, Z, "parse_mesh")
    common = ["--mesh", str(tmp_path / "mesh.h5"), "--metrics", str(tmp_path / "metrics.h5"), "--dt", "1e-3"]
    a = tmp_path / "a"
    assert run.main(common + ["--out", str(a), "--time", "0.025", "--step-plt", "10", "--chk-out", "--step-chk",
                              "20", "--average", "--avg-step", "5", "--avg-total", "2"]) == 0
    for f in ("PLT/plt-10.h5", "PLT/plt-10.xmf", "PLT/plt-20.h5", "PLT/plt-25.h5", "CHK/chk-20.h5",
              "CHK/chk-25.h5", "AVG/avg-10.h5"):
        assert os.path.exists(a / f), f
    p25 = h5.read(str(a / "PLT/plt-25.h5"))
    assert all(np.isfinite(v).all() for v in p25.values())
    # the free stream at the inflow, the no-slip wall pulling u down next to it
    assert p25["u"][:, 0, :].mean() < p25["u"][:, -1, :].mean()
    avg = h5.read(str(a / "AVG/avg-10.h5"))["avg"]
    assert avg.shape == (6, 8, 20, 24) and np.isfinite(avg).all()
    # restart from the checkpoint of step 20 for 5 steps: as steps 21-25 of the first run,
    # but from the Float32 primitives of the file. Time 0.0055: in Float32, 5 dt lies just
    # above 0.005, where the reference's loop would stop after 4 steps
    assert run.n_steps(1e-3, 0.0055, 200000) == 5 and run.n_steps(1e-3, 0.005, 200000) == 4
    b = tmp_path / "b"
    assert run.main(common + ["--out", str(b), "--time", "0.0055", "--restart", str(a / "CHK/chk-20.h5")]) == 0
    Qa = files.read_checkpoint(str(a / "CHK/chk-25.h5")).astype(np.float64)
    pb = h5.read(str(b / "PLT/plt-5.h5"))
    I = (slice(4, -4),) * 3
    vel = np.abs(Qa[1:4][(slice(None),) + I]).max()  # one scale for u, v, w
    for n, name in enumerate(files.PRIM_NAMES):
        scale = vel if name in ("u", "v", "w") else np.abs(Qa[n][I]).max()
        assert np.abs(pb[name] - Qa[n][I]).max() <= 1e-5 * scale, name

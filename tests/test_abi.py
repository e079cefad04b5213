"""CPU tests of the C ABI and the host logic: every symbol the header declares is exported,
the ctypes structures match the C layout, the Python defaults match the library's (and
run.jl's), and the multi-rank aggregation of bench.py works with two gloo ranks. No
kernel is launched."""
import ctypes as C
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "flame3d_gpu.h"


@pytest.fixture(scope="module")
def lib():
    from flame3d_mhd_gb300 import abi, build
    build.build()
    return abi.load()


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(f3d_\w+)\s*\(", text, flags=re.M)))


def test_header_declarations_are_exported(lib):
    from flame3d_mhd_gb300 import abi
    decl = declared_functions()
    assert len(decl) >= 25
    assert sorted(abi.EXPORTED) == decl
    for name in decl:
        assert hasattr(lib, name), name
    nm = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True, text=True)
    if nm.returncode == 0:
        syms = set(re.findall(r"\bT (f3d_\w+)", nm.stdout))
        assert set(decl) <= syms


def test_struct_layout_matches_header(tmp_path):
    """sizeof/offsetof of f3d_params and f3d_bc from the C compiler vs ctypes."""
    from flame3d_mhd_gb300.abi import F3DBc, F3DParams
    fields = [f for f, _ in F3DParams._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {",
             'printf("%zu %zu\\n", sizeof(f3d_params), sizeof(f3d_bc));']
    lines += [f'printf("%zu\\n", offsetof(f3d_params, {f}));' for f in fields]
    lines += ["return 0; }"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-O0", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == C.sizeof(F3DParams)
    assert int(out[1]) == C.sizeof(F3DBc)
    for f, off in zip(fields, out[2:]):
        assert getattr(F3DParams, f).offset == int(off), f


def test_default_params_match_library_and_run_jl(lib):
    from flame3d_mhd_gb300 import abi
    p_lib = abi.F3DParams()
    assert lib.f3d_default_params(64, 32, 16, C.byref(p_lib)) == abi.F3D_OK
    p_py = abi.make_params(64, 32, 16)
    assert bytes(p_lib) == bytes(p_py)
    # run.jl:8-13, 61, 68-73; boundary.jl free stream and BC kinds
    assert (p_py.gamma, p_py.rg, p_py.c_s, p_py.t_s, p_py.pr) == (1.4, 287.0, 1.458e-6, 110.4, 0.72)
    assert (p_py.phi1, p_py.phi2, p_py.phi3, p_py.linear_phi) == (0.05, 1.0, 10.0, 1.0)
    assert (p_py.split_method, p_py.character, p_py.viscous) == (abi.SPLIT_SW, 1, 1)
    kinds = [b.kind for b in p_py.bc]
    assert kinds == [abi.BC_DIRICHLET, abi.BC_ZERO_GRADIENT, abi.BC_WALL_ADIABATIC, abi.BC_DIRICHLET,
                     abi.BC_PERIODIC, abi.BC_PERIODIC]
    assert p_py.bc[0].u == 0.5 and abs(p_py.bc[0].p - 1 / 1.4) < 1e-15


def test_version(lib):
    assert lib.f3d_version() == 10000


def test_cases_shapes():
    from flame3d_mhd_gb300 import cases
    c = cases.sod(16, 8, 8)
    assert c["Q"].shape == (6, 16, 16, 24)
    assert c["x"].shape == (16, 16, 24)
    assert c["dt"] > 0
    t = cases.tgv(8)
    assert t["params"].phi3 == float("inf")


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    v = bench.reduce_max(10.0 + rank)
    with open(out / f"r{rank}", "w") as f:
        f.write(repr(v))
    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks(tmp_path):
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_rank_main, args=(2, port, tmp_path), nprocs=2, join=True, start_method="spawn")
    assert float((tmp_path / "r0").read_text()) == 11.0
    assert float((tmp_path / "r1").read_text()) == 11.0


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""

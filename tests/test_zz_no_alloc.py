"""f3d_rhs_noalloc: the RHS for callers that cannot allocate device memory.

Such callers (code running inside a CUDA-graph stream capture, or hosts whose memory pool
owns the device and forbids cudaMalloc/cudaFree) get the RHS without a context: the
entry point keeps its scratch in a fixed device array of the library. This test calls it
through the C ABI twice in a row, on two different grids and states, and checks each result
against the context-based f3d_rhs at the parity tolerance. The array keeps the previous
call's contents, so the second call also shows that nothing stale leaks into a result.
The file is collected last so that a run stopping at the first failure has run the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300 import abi, cases
from flame3d_mhd_gb300.abi import BC_PERIODIC, make_params
from flame3d_mhd_gb300.solver import Flame3D
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the RHS parity tolerance of tests/test_gpu_parity.py
NG = 4


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _viscous_hybrid_inputs():
    """24x16x12 curvilinear grid, reference boundary conditions, viscous, hybrid scheme."""
    P = make_params(24, 16, 12, rg=1.0, c_s=1e-2, t_s=1.0, phi1=0.02, phi2=0.1, phi3=0.4)
    s = (P.nz + 8, P.ny + 8, P.nx + 8)
    ax = [(np.arange(n) - NG + 0.5) / (n - 8) for n in s]
    Z, E, X = np.meshgrid(*ax, indexing="ij")
    tp = 2 * np.pi
    x = X + 0.03 * np.sin(tp * E) * np.sin(tp * Z)
    y = E + 0.03 * np.sin(tp * Z) * np.sin(tp * X)
    z = Z + 0.03 * np.sin(tp * X) * np.sin(tp * E)
    rng = np.random.default_rng(21)
    Q = np.zeros((6, *s))
    Q[0] = 1.0 + 0.1 * rng.uniform(-1, 1, s)
    Q[1:4] = 0.2 * rng.uniform(-1, 1, (3, *s))
    Q[4] = (1.0 + 0.1 * rng.uniform(-1, 1, s)) / 1.4
    Q[4, 8, 9, 10] *= 50.0
    Q[5] = Q[4] / Q[0]
    return P, Q, x, y, z


def _sod_inputs():
    c = cases.sod(32, 16, 16)
    return c["params"], c["Q"], c["x"], c["y"], c["z"]


def _rhs_both(lib, P, Q0, x, y, z):
    m, J, Q, _ = orc.prepare(P, Q0, x, y, z)
    md, Jd, Qd = [_dev(a) for a in m], _dev(J), _dev(Q)
    out = torch.zeros((5, *Q.shape[1:]), dtype=torch.float64, device="cuda")
    arr = (C.c_void_p * 9)(*[C.c_void_p(a.data_ptr()) for a in md])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.f3d_rhs_noalloc(C.byref(P), arr, C.c_void_p(Jd.data_ptr()), C.c_void_p(Qd.data_ptr()),
                             C.c_void_p(out.data_ptr()), stream)
    assert rc == abi.F3D_OK
    ref_solver = Flame3D(P)
    ref_solver.set_metrics(md, Jd)
    ref = ref_solver.rhs(Qd)
    torch.cuda.synchronize()
    ref_solver.close()
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    return out.cpu().numpy()[I], ref.cpu().numpy()[I]


def test_rhs_noalloc_matches_rhs_twice(gpu_lib):
    lib = gpu_lib
    for make in (_viscous_hybrid_inputs, _sod_inputs):
        got, ref = _rhs_both(lib, *make())
        assert np.isfinite(got).all()
        assert rel_linf(got, ref) <= TOL


def test_rhs_noalloc_rejects_large_grid(gpu_lib):
    P = make_params(64, 64, 64, bc=[dict(kind=BC_PERIODIC)] * 6)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    rc = gpu_lib.f3d_rhs_noalloc(C.byref(P), (C.c_void_p * 9)(*[p] * 9), p, p, p, None)
    assert rc == abi.F3D_ERR_TOO_LARGE

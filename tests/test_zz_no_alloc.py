"""f3d_rhs_noalloc: the RHS for callers that cannot allocate device memory.

Such callers (a host whose memory pool has reserved the device's memory and forbids
foreign cudaMalloc/cudaFree, or a loop that cannot afford cudaFree's device-wide
synchronisation) get the RHS without a context: the entry point keeps its scratch in a fixed
device array of the library. This test calls it through the C ABI three times in a row:
two viscous grids of different sizes and states, then an inviscid shock tube. Each result is
checked against the CPU oracle at the RHS parity tolerance (as tests/test_gpu_parity.py
states it) and against the context-based f3d_rhs. The array keeps
the previous call's contents, and the second viscous call reads viscous-flux scratch the
first one left behind at other offsets, so a stale value would show in its result. The file
is collected last so that a run stopping at the first failure has run the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import assert_rhs_parity, rel_linf, rhs_parity
from flame3d_mhd_gb300 import abi, cases
from flame3d_mhd_gb300.abi import BC_PERIODIC, make_params
from flame3d_mhd_gb300.solver import Flame3D
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the RHS parity tolerance of tests/test_gpu_parity.py
NG = 4


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _viscous_hybrid_inputs(n=(24, 16, 12), seed=21, amp=0.03):
    """Curvilinear grid, reference boundary conditions, viscous, hybrid scheme."""
    P = make_params(*n, viscous=1, rg=1.0, c_s=1e-2, t_s=1.0, phi1=0.02, phi2=0.1, phi3=0.4)
    s = (P.nz + 8, P.ny + 8, P.nx + 8)
    ax = [(np.arange(k) - NG + 0.5) / (k - 8) for k in s]
    Z, E, X = np.meshgrid(*ax, indexing="ij")
    tp = 2 * np.pi
    x = X + amp * np.sin(tp * E) * np.sin(tp * Z)
    y = E + amp * np.sin(tp * Z) * np.sin(tp * X)
    z = Z + amp * np.sin(tp * X) * np.sin(tp * E)
    rng = np.random.default_rng(seed)
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


def _noalloc_call(lib, P, Q0, x, y, z):
    """f3d_rhs_noalloc through the C ABI; returns its interior result, f3d_rhs's, and the
    oracle-prepared inputs."""
    m, J, Q, _ = orc.prepare(P, Q0, x, y, z)
    md, Jd, Qd = [_dev(a) for a in m], _dev(J), _dev(Q)
    out = torch.full((5, *Q.shape[1:]), float("nan"), dtype=torch.float64, device="cuda")
    arr = (C.c_void_p * 9)(*[C.c_void_p(a.data_ptr()) for a in md])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.f3d_rhs_noalloc(C.byref(P), arr, C.c_void_p(Jd.data_ptr()), C.c_void_p(Qd.data_ptr()),
                             C.c_void_p(out.data_ptr()), stream)
    assert rc == abi.F3D_OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref_solver = Flame3D(P)
    ref_solver.set_metrics(md, Jd)
    ref = ref_solver.rhs(Qd)
    torch.cuda.synchronize()
    ref_solver.close()
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    return got[I], ref.cpu().numpy()[I], (P, Q, m, J)


def _check_against_oracle(got, inputs):
    """The RHS parity bar of tests/test_gpu_parity.py (conftest.assert_rhs_parity)."""
    P, Q, m, J = inputs
    full = np.zeros((5, *Q.shape[1:]))
    full[:, NG:-NG, NG:-NG, NG:-NG] = got
    assert_rhs_parity(rhs_parity(P, Q, m, J, full))


def test_rhs_noalloc_three_calls_in_a_row(gpu_lib):
    lib = gpu_lib
    runs = [lambda: _viscous_hybrid_inputs((24, 16, 12), 21, 0.03),
            lambda: _viscous_hybrid_inputs((20, 12, 16), 22, 0.05),  # other grid: other offsets
            _sod_inputs]
    for make in runs:
        got, ref, inputs = _noalloc_call(lib, *make())
        assert np.isfinite(got).all()
        _check_against_oracle(got, inputs)
        assert rel_linf(got, ref) <= TOL


def test_rhs_noalloc_rejects_large_grid(gpu_lib):
    P = make_params(64, 64, 64, bc=[dict(kind=BC_PERIODIC)] * 6)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    rc = gpu_lib.f3d_rhs_noalloc(C.byref(P), (C.c_void_p * 9)(*[p] * 9), p, p, p, None)
    assert rc == abi.F3D_ERR_TOO_LARGE

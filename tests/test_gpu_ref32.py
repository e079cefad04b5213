"""F3D_PREC_REF32: the reference's Float32 arrays and arithmetic, against the oracle's
Float32 restatement of the same formulas (orc32_*: Float32 everywhere, WENO7 weights in
FP64, as schemes.jl:178-185).

Tolerances, written per check:
- c2Prim, prim2c and the ghost rules: bitwise (the same IEEE Float32 operations in the
  same order, no contraction on either side);
- one RHS, as error relative to the flux scale (max over cells of J * sum |face fluxes|
  of the RHS differences, per variable): GPU against the extended-precision RHS within
  1.5x the oracle's own Float32 error plus 2e-6 (as accurate as the reference's Float32
  arithmetic), and GPU against the oracle's Float32 RHS within twice that error (two
  evaluations of the same Float32 formulas, rounded differently: the GPU contracts
  multiply-adds in the reconstruction and differences the faces in another order);
- five RK3 steps, each variable relative to its largest magnitude: against the FP64
  trajectory of the same inputs no further than 4x the oracle's own Float32 trajectory
  plus 1e-6, and against that Float32 trajectory within 4x its distance to FP64 plus
  1e-6 (measured: 6.1e-7 vs 5.7e-7 inviscid periodic; 4.8e-6 vs 1.6e-6 on the viscous
  wall case, where the per-variable maximum sits on the smallest momentum component and
  the two Float32 roundings of 15 stages part by a few ulps of the largest flux);
  stage-by-stage stepping equal to the captured steps bitwise.
"""
import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300.abi import (BC_DIRICHLET, BC_PERIODIC, BC_WALL_ADIABATIC, BC_WALL_ISOTHERMAL,
                                   BC_ZERO_GRADIENT, F3D_ERR_ARG, F3D_ERR_UNSUPPORTED, PREC_REF32, F3DError,
                                   make_params)
from flame3d_mhd_gb300.cases import params_copy
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc
from test_gpu_parity import curvilinear_coords, random_state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
f32 = np.float32


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


PER, ZG = dict(kind=BC_PERIODIC), dict(kind=BC_ZERO_GRADIENT)
FS = dict(kind=BC_DIRICHLET, rho=1.1, u=0.4, v=0.05, w=-0.02, p=0.8)
BCS = {
    "periodic": [PER] * 6,
    # t_wall above half the hottest cell (pressure spikes reach T ~ 170 at Rg = 1): T_g = 2 T_w - T > 0
    "walls": [ZG, ZG, dict(kind=BC_WALL_ISOTHERMAL, t_wall=100.0), FS, PER, PER],
    "mixed": [FS, dict(kind=BC_WALL_ADIABATIC), PER, PER, ZG, FS],
    # a wall at the state's own temperature (0.5-1.1 without spikes at Rg = 1)
    "walls_mild": [ZG, ZG, dict(kind=BC_WALL_ISOTHERMAL, t_wall=0.8), FS, PER, PER],
}


def _case(bcs="periodic", seed=41, spikes=20, n=(24, 16, 12), **kw):
    kw.setdefault("phi1", 0.02)
    kw.setdefault("phi2", 0.1)
    kw.setdefault("phi3", 0.4)
    if kw.get("viscous"):
        kw.update(rg=1.0, c_s=1e-2, t_s=1.0)
    P64 = make_params(*n, bc=BCS[bcs], **kw)
    x, y, z = curvilinear_coords(P64)
    Q0 = random_state(P64, seed, spikes)
    if kw.get("viscous"):  # T at the interior (the ghosts are filled by the oracle below)
        I = (slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
        Q0[5][I] = Q0[4][I] / (Q0[0][I] * P64.rg)
    m, J, Q, U = orc.prepare(P64, Q0, x, y, z)
    P = params_copy(P64, precision=PREC_REF32)
    m32, J32, U32 = [a.astype(f32) for a in m], J.astype(f32), U.astype(f32)
    # the Float32 state the reference would hold: c2Prim and the ghost rules in Float32
    Q32 = orc.c2prim32(P, U32)
    orc.fill_ghosts32(P, Q32, U32)
    s = Flame3D(P)
    keep = ([dev(a) for a in m32], dev(J32))
    s.set_metrics(*keep)
    return P, P64, (m, J, Q, U), (m32, J32, Q32, U32), s, keep


def test_pointwise_bitwise(gpu_lib):
    for bcs in ("periodic", "walls", "mixed"):
        P, P64, _, (m32, J32, Q32, U32), s, keep = _case(bcs)
        Ud = dev(U32)
        Qd = torch.zeros_like(dev(Q32))
        s.c2Prim(Ud, Qd)
        Qo = orc.c2prim32(P, U32)
        assert np.array_equal(host(Qd)[I], Qo[I]), bcs
        # ghost rules from scrambled ghosts, Q and U
        rng = np.random.default_rng(3)
        g = np.ones(Q32.shape[1:], bool)
        g[NG:-NG, NG:-NG, NG:-NG] = False
        Qi, Ui = Q32.copy(), U32.copy()
        Qi[:, g] = rng.uniform(-5, 5, (6, g.sum())).astype(f32)
        Ui[:, g] = rng.uniform(-5, 5, (5, g.sum())).astype(f32)
        Qd, Ud = dev(Qi), dev(Ui)
        s.fillGhost(Qd, Ud)
        orc.fill_ghosts32(P, Qi, Ui)
        assert np.array_equal(host(Qd), Qi), bcs
        assert np.array_equal(host(Ud), Ui), bcs
        U2 = torch.zeros_like(Ud)
        s.prim2c(U2, dev(Q32))
        assert np.array_equal(host(U2), orc.prim2c32(P, Q32)), bcs
        s.close()


@pytest.mark.parametrize("bcs,character,viscous,les", [("periodic", 1, 0, 0), ("periodic", 0, 0, 0), ("walls", 1, 1, 0),
                                                       ("mixed", 0, 1, 0), ("walls", 1, 1, 1), ("mixed", 0, 1, 2)])
def test_rhs_against_the_reference_arithmetic(gpu_lib, bcs, character, viscous, les):
    """les: Smagorinsky (1) or WALE (2) eddy viscosity in the Float32 viscous fluxes."""
    P, P64, (m, J, Q, U), (m32, J32, Q32, U32), s, keep = _case(bcs, character=character, viscous=viscous, les=les)
    r = host(s.rhs(dev(Q32))).astype(np.float64)
    r32 = orc.rhs32(P, Q32, m32, J32).astype(np.float64)
    Q64 = Q32.astype(np.float64)
    rl, scale = orc.rhs_ld(P64, Q64, [a.astype(np.float64) for a in m32], J32.astype(np.float64))
    gpu_orc = max(float(np.abs(r[n][I[1:]] - r32[n][I[1:]]).max() / scale[n]) for n in range(5))
    gpu_ld = max(float(np.abs(r[n][I[1:]] - rl[n][I[1:]]).max() / scale[n]) for n in range(5))
    orc_ld = max(float(np.abs(r32[n][I[1:]] - rl[n][I[1:]]).max() / scale[n]) for n in range(5))
    msg = f"gpu-vs-orc32 {gpu_orc:.2e} gpu-vs-ld {gpu_ld:.2e} orc32-vs-ld {orc_ld:.2e}"
    print(msg)
    assert gpu_orc <= max(2e-6, 2.0 * orc_ld), msg
    assert gpu_ld <= 1.5 * orc_ld + 2e-6, msg
    if les:  # the eddy viscosity moves the answer far beyond the bars above (2e-4 .. 4e-4)
        r0 = orc.rhs32(params_copy(P, les=0), Q32, m32, J32).astype(np.float64)
        assert max(float(np.abs(r32[n][I[1:]] - r0[n][I[1:]]).max() / scale[n]) for n in range(5)) > 2e-5
    s.close()


@pytest.mark.parametrize("bcs,viscous", [("periodic", 0), ("walls_mild", 1)])
def test_rk3_steps_against_the_reference_arithmetic(gpu_lib, bcs, viscous):
    P, P64, (m, J, Q, U), (m32, J32, Q32, U32), s, keep = _case(bcs, viscous=viscous, spikes=0)
    dt, steps = 2e-4, 5
    Ud, Und, Qd = dev(U32), dev(np.zeros_like(U32)), dev(Q32)
    with side_stream():
        s.time_step(Ud, Und, Qd, dt, steps)
    torch.cuda.synchronize()
    Uo, Uno, Qo = U32.copy(), np.zeros_like(U32), Q32.copy()
    orc.rk3_32(P, steps, dt, Uo, Uno, Qo, m32, J32)
    Ug = host(Ud)
    assert np.isfinite(Ug).all()
    d = rel_linf(Ug[I].astype(np.float64), Uo[I].astype(np.float64))
    # the FP64 trajectory of the same Float32 inputs
    U64, Un64, Q64 = U32.astype(np.float64), np.zeros(U32.shape), Q32.astype(np.float64)
    m64, J64 = [a.astype(np.float64) for a in m32], J32.astype(np.float64)
    orc.rk3(P64, steps, dt, U64, Un64, Q64, m64, J64)
    gpu64 = rel_linf(Ug[I].astype(np.float64), U64[I])
    orc64 = rel_linf(Uo[I].astype(np.float64), U64[I])
    msg = f"gpu-vs-orc32 {d:.2e} gpu-vs-fp64 {gpu64:.2e} orc32-vs-fp64 {orc64:.2e}"
    print(msg)
    assert gpu64 <= 4.0 * orc64 + 1e-6, msg
    assert d <= 4.0 * orc64 + 1e-6, msg
    # one stage at a time gives the same state as the captured steps
    Ud2, Und2, Qd2 = dev(U32), dev(np.zeros_like(U32)), dev(Q32)
    for _ in range(steps):
        for st in (1, 2, 3):
            s.rk3_stage(st, dt, Ud2, Und2, Qd2)
    torch.cuda.synchronize()
    assert torch.equal(Ud2, Ud)
    s.close()


def test_ref32_entry_errors(gpu_lib):
    P, P64, _, (m32, J32, Q32, U32), s, keep = _case()
    # FP64-array entries refuse the Float32 context, and the reverse
    rc = s.lib.f3d_rhs(s._h, dev(Q32.astype(np.float64)).data_ptr(), dev(U32.astype(np.float64)).data_ptr(), None)
    assert rc == F3D_ERR_ARG
    s64 = Flame3D(P64)
    rc = s64.lib.f3d_rhs_f32(s64._h, dev(Q32).data_ptr(), dev(U32).data_ptr(), None)
    assert rc == F3D_ERR_ARG
    s64.close()
    with pytest.raises(TypeError):
        s.rhs(dev(Q32.astype(np.float64)))
    for kw in (dict(lts=1, lts_cfl=0.5), dict(filter=1)):
        with pytest.raises(F3DError) as e:
            Flame3D(params_copy(P, **kw))
        assert e.value.code == F3D_ERR_UNSUPPORTED
    s.close()


@pytest.mark.parametrize("pipeline", ["readfort", "parse_mesh"])
def test_set_up_metrics_bitwise(gpu_lib, tmp_path, pipeline):
    """f3d_compute_metrics_f32 equals the reference's Float32 set-up metrics bit for bit:
    the swept ramp through readfort.jl's pipeline (OCFD file, Float32, ghosts, metres) and the
    flat plate of parse_mesh.jl."""
    from flame3d_mhd_gb300 import meshgen
    from flame3d_mhd_gb300.abi import METRICS_PARSE_MESH, METRICS_READFORT
    from flame3d_mhd_gb300.grid import mesh_from_ocfd, write_ocfd_mesh
    if pipeline == "readfort":
        q = dict(nx=64, ny=24, nz=6, nprocs=1, nx_inlet=40, nx_corner=20, nx_buff=4, dx_inlet=0.9, lx_inlet=30.0,
                 lx_corner=8.0, alfax_buff=1.05, sw_angle=20.0, comp_angle=24.0, high=6.0, hy_wall=0.01, lz=3.0)
        path = str(tmp_path / "OCFD3d-Mesh.dat")
        write_ocfd_mesh(path, *meshgen.swept_ramp_mesh(q))
        X, Y, Z = mesh_from_ocfd(path, q["nx"], q["ny"], q["nz"])
        n, coef = (q["nx"], q["ny"], q["nz"]), METRICS_READFORT
    else:
        n = (24, 20, 8)
        X, Y, Z = meshgen.flat_plate_grid(*n)
        coef = METRICS_PARSE_MESH
    s = Flame3D(params_copy(make_params(*n), precision=PREC_REF32))
    ms, J = s.compute_metrics(dev(X), dev(Y), dev(Z), coef)
    mr, Jr = meshgen.metrics_f32(X, Y, Z, pipeline)
    assert np.array_equal(host(J), Jr)
    for a, b in zip(ms, mr):
        assert np.array_equal(host(a), b)
    s.set_metrics(ms, J)  # usable as the context's metrics
    with pytest.raises(F3DError):
        s.compute_metrics(dev(X), dev(Y), dev(Z), 7)
    s.close()

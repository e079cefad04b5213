"""Finite-volume RHS (FVM.jl, the reference's default scheme) on the GPU against the oracle:
face fluxes of both reconstructions per direction, the full RHS (with viscous terms), and
graph-captured RK3 steps.

Tolerances: face fluxes and RHS within 1e-12 of the oracle relative to each variable's
largest magnitude, unless the FP64 oracle itself is further than that from the long-double
evaluation of the same formulas (then within 3x the oracle's own error, and the GPU within
2x of the oracle's distance to long double, as the finite-difference parity tests); states
after RK3 steps within 1e-12 of the largest state component. Face normals are computed in
the oracle's operation order without FMA contraction, so the characteristic tangent basis
(which switches at |nz| = |ny|) is the oracle's at every face."""
import numpy as np
import pytest
import torch

from conftest import rel_linf
from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import (BC_PERIODIC, F3D_ERR_STATE, F3D_ERR_UNSUPPORTED, PREC_MIXED, SCHEME_FVM_CONS,
                                   SCHEME_FVM_EIGEN, F3DError, make_params)
from flame3d_mhd_gb300.cases import params_copy
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc
from test_oracle_fvm import _coords, _state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
SCHEMES = {"eigen": SCHEME_FVM_EIGEN, "cons": SCHEME_FVM_CONS}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def _case(scheme, viscous=0, n=(20, 14, 12), bc="periodic", seed=21):
    kw = dict(viscous=viscous, phi1=0.02, phi2=0.1, phi3=0.4, scheme=SCHEMES[scheme])
    if viscous:
        kw.update(rg=1.0, c_s=1e-2, t_s=1.0)
    if bc == "periodic":
        kw["bc"] = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(*n, **kw)
    x, y, z = _coords(P, 0.02)
    Q0 = _state(P, seed, spikes=15, noise=0.03)
    if viscous:
        Q0[5] = Q0[4] / (Q0[0] * P.rg)
    m, J, Q, U = orc.prepare(P, Q0, x, y, z)
    return P, x, y, z, m, J, Q, U


def _solver(P, x, y, z, m, J):
    s = Flame3D(P)
    s.set_metrics([dev(a) for a in m], dev(J))
    s.set_coordinates(dev(x), dev(y), dev(z))
    return s


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_fvm_face_flux_parity(gpu_lib, scheme):
    P, x, y, z, m, J, Q, U = _case(scheme)
    s = _solver(P, x, y, z, m, J)
    phi = orc.sensor(P, Q)
    Uq = orc.prim2c(P, Q)  # the RHS entry reconstructs from prim2c(Q)
    for d in range(3):
        S = orc.metric_norm(P, m[3 * d], m[3 * d + 1], m[3 * d + 2])
        Fo = orc.fvm_face_flux(P, d, scheme == "eigen", phi, S, Q, Uq, x, y, z)
        Fd = torch.zeros((5, *orc.face_shape(P, d)), dtype=torch.float64, device="cuda")
        s.advect(d, Fd, dev(phi), dev(Q))
        Fg = host(Fd)
        assert rel_linf(Fg, Fo) <= 1e-12, (d, rel_linf(Fg, Fo))
    s.close()


@pytest.mark.parametrize("scheme,viscous", [("eigen", 0), ("cons", 0), ("eigen", 1)])
def test_fvm_rhs_parity(gpu_lib, scheme, viscous):
    P, x, y, z, m, J, Q, U = _case(scheme, viscous)
    s = _solver(P, x, y, z, m, J)
    r = host(s.rhs(dev(Q)))
    orc.set_coordinates(x, y, z)
    try:
        ro = orc.rhs(P, Q, m, J)
        rl, _ = orc.rhs_ld(P, Q, m, J)
    finally:
        orc.set_coordinates(None)
    plain, gpu_ld, orc_ld = rel_linf(r[I], ro[I]), rel_linf(r[I], rl[I]), rel_linf(ro[I], rl[I])
    msg = f"plain {plain:.2e} gpu-vs-ld {gpu_ld:.2e} oracle-vs-ld {orc_ld:.2e}"
    assert plain <= max(1e-12, 3.0 * orc_ld), msg
    assert gpu_ld <= max(1e-12, 2.0 * orc_ld), msg
    s.close()


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_fvm_rk3_steps_parity(gpu_lib, scheme):
    P, x, y, z, m, J, Q, U = _case(scheme, viscous=0)
    s = _solver(P, x, y, z, m, J)
    dt, steps = 2e-3, 5
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream():
        s.time_step(Ud, Und, Qd, dt, steps)
    torch.cuda.synchronize()
    orc.set_coordinates(x, y, z)
    try:
        Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
        orc.rk3(P, steps, dt, Uo, Uno, Qo, m, J)
    finally:
        orc.set_coordinates(None)
    assert rel_linf(host(Ud)[I], Uo[I], per_var=False) <= 1e-12
    s.close()


def test_fvm_sod_reference_bcs_steps(gpu_lib):
    """The reference's default configuration (run.jl: finite_volume, eigen_reconstruction)
    on the shock tube with zero-gradient x and periodic y, z. The interface is planar: on
    this coarse curvilinear grid the perturbed interface leaves two-cell valleys of the
    light state in the eta / zeta stencils, where FVM.jl's WENO5 of the conserved variables
    reconstructs a negative density and the HLLC speeds become NaN (the oracle and the GPU
    both propagate it, as the reference does; tested below)."""
    c = cases.sod(48, 12, 12, amp=0.0)
    P = params_copy(c["params"], scheme=SCHEME_FVM_EIGEN)
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    s = _solver(P, c["x"], c["y"], c["z"], m, J)
    Ud, Und, Qd = dev(U), dev(np.zeros_like(U)), dev(Q)
    with side_stream():
        s.time_step(Ud, Und, Qd, c["dt"], 10)
    torch.cuda.synchronize()
    orc.set_coordinates(c["x"], c["y"], c["z"])
    try:
        Uo, Uno, Qo = U.copy(), np.zeros_like(U), Q.copy()
        orc.rk3(P, 10, c["dt"], Uo, Uno, Qo, m, J)
        Ul, Unl, Ql = U.copy(), np.zeros_like(U), Q.copy()
        orc.rk3_ld(P, 10, c["dt"], Ul, Unl, Ql, m, J)
    finally:
        orc.set_coordinates(None)
    Ug = host(Ud)
    assert np.isfinite(Ug).all()
    # across the shock the FP64 trajectory itself drifts from the extended-precision one;
    # the GPU must be as close to that as the FP64 oracle is
    gpu_ld = rel_linf(Ug[I], Ul[I], per_var=False)
    orc_ld = rel_linf(Uo[I], Ul[I], per_var=False)
    plain = rel_linf(Ug[I], Uo[I], per_var=False)
    msg = f"plain {plain:.2e} gpu-vs-ld {gpu_ld:.2e} oracle-vs-ld {orc_ld:.2e}"
    assert gpu_ld <= max(1e-12, 3.0 * orc_ld), msg
    assert plain <= max(1e-12, 4.0 * orc_ld), msg
    s.close()


def test_fvm_negative_density_propagates_nan(gpu_lib):
    """The coarse curvilinear shock tube: FVM.jl's scheme reconstructs a negative density at
    a few eta / zeta faces, and the RHS is NaN there on the GPU as in the oracle (Julia's
    min / max propagate NaN); the non-finite check reports it."""
    c = cases.sod(48, 12, 12)
    P = params_copy(c["params"], scheme=SCHEME_FVM_CONS)
    m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    s = _solver(P, c["x"], c["y"], c["z"], m, J)
    r = host(s.rhs(dev(Q)))
    orc.set_coordinates(c["x"], c["y"], c["z"])
    try:
        ro = orc.rhs(P, Q, m, J)
    finally:
        orc.set_coordinates(None)
    bad_o = ~np.isfinite(ro[I])
    assert bad_o.any()
    assert np.array_equal(~np.isfinite(r[I]), bad_o)
    fin = ~bad_o
    assert np.abs(r[I][fin] - ro[I][fin]).max() <= 1e-12 * np.abs(ro[I][fin]).max()
    assert not s.check_finite(dev(ro))
    s.close()


def test_fvm_errors(gpu_lib):
    P = make_params(8, 8, 8, scheme=SCHEME_FVM_EIGEN)
    with pytest.raises(F3DError) as e:
        Flame3D(params_copy(P, precision=PREC_MIXED))
    assert e.value.code == F3D_ERR_UNSUPPORTED
    s = Flame3D(P)
    s.set_metrics([s.field(1) for _ in range(9)], s.field(1))
    with pytest.raises(F3DError) as e:
        s.rhs(s.field(6))  # coordinates not set
    assert e.value.code == F3D_ERR_STATE
    s.close()


def _jl_fvm_cases():
    """The finite-volume cases of tests/golden/jl_reference_rhs.npz: FVM.jl translated
    mechanically (two defects corrected, oracle/ref_jl/jl2py.py CORRECTIONS) and evaluated in
    binary64, with the inputs it was computed from."""
    import json
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "jl_reference_rhs.npz", allow_pickle=True)
    out = {}
    for name in sorted({k.split("__")[0] for k in d.files if k.endswith("__rhs_fvm")}):
        meta = json.loads(str(d[f"{name}__meta"]))
        P = make_params(*meta["n"], **meta["params"])
        steps = None
        if f"{name}__U_rk3_fvm" in d.files:
            rk = json.loads(str(d["provenance"]))["rk3"]
            steps = (d[f"{name}__U_rk3_fvm"], rk["dt"], rk["steps"])
        out[name] = (P, d[f"{name}__Q"], [d[f"{name}__{a}"] for a in "xyz"],
                     [d[f"{name}__F{k}"] for k in range(3)], d[f"{name}__rhs_fvm"], steps)
    return out


@pytest.mark.parametrize("name", sorted(_jl_fvm_cases()))
def test_fvm_against_the_translated_reference(gpu_lib, name):
    """Face fluxes, the RHS and (boundary.jl's boundary set) two SSP-RK3 steps of the GPU's
    finite-volume path against the reference's own on the same inputs (faces of all four
    branches). Faces and RHS: the bar of the tests above, within max(1e-12, 3x) the FP64
    reference's own distance to the long-double evaluation (on the FP64 face geometry) and
    the GPU within 2x that distance of long double, relative to each variable's largest
    magnitude; states within 1e-12 of the largest component."""
    P, Q, (x, y, z), Fref, rref, steps = _jl_fvm_cases()[name]
    m, J = orc.metrics(P, x, y, z)  # equal to the reference's metrics bit for bit
    s = _solver(P, x, y, z, m, J)
    phi, Uq = orc.sensor(P, Q), orc.prim2c(P, Q)
    eigen = int(P.scheme) == SCHEME_FVM_EIGEN

    def check(g, ref, ld, what):
        plain, gpu_ld, ref_ld = rel_linf(g, ref), rel_linf(g, ld), rel_linf(ref, ld)
        msg = f"{what}: plain {plain:.2e} gpu-vs-ld {gpu_ld:.2e} reference-vs-ld {ref_ld:.2e}"
        assert plain <= max(1e-12, 3.0 * ref_ld), msg
        assert gpu_ld <= max(1e-12, 2.0 * ref_ld), msg

    for d in range(3):
        Fd = torch.zeros((5, *orc.face_shape(P, d)), dtype=torch.float64, device="cuda")
        s.advect(d, Fd, dev(phi), dev(Q))
        S = orc.metric_norm(P, m[3 * d], m[3 * d + 1], m[3 * d + 2])
        check(host(Fd), Fref[d], orc.fvm_face_flux_ld(P, d, eigen, phi, S, Q, Uq, x, y, z), f"faces {d}")
    r = host(s.rhs(dev(Q)))
    orc.set_coordinates(x, y, z)
    try:
        rl, _ = orc.rhs_ld(P, Q, m, J)
    finally:
        orc.set_coordinates(None)
    check(r[I], rref[I], rl[I], "rhs")
    if steps is not None:
        Uref, dt, n = steps
        Ud, Und, Qd = dev(Uq), dev(np.zeros_like(Uq)), dev(Q)
        with side_stream():
            s.time_step(Ud, Und, Qd, dt, n)
        torch.cuda.synchronize()
        assert rel_linf(host(Ud)[I], Uref[I], per_var=False) <= 1e-12
    s.close()

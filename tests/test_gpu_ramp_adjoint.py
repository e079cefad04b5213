"""Adjoint pieces of the compression-ramp study: the inflow-profile cotangent of the RHS and
step VJPs against the oracle's dual-number derivative with respect to the profile, the stage
outputs of f3d_rk3_step_vjp_stages, the memory-bounded reversal against the sqrt(N)
checkpoints, and the whole gradient of the windowed wall-pressure force with respect to the
inflow velocity scalings and the ramp angle against central differences on a reduced grid.

Tolerances, written per check:
- dot products <profile_bar, d> = <L_bar, dL/dprofile . d>: 1e-10 relative to the sum of
  |terms| (both sides exact derivatives of the same branch-frozen FP64 scheme); with WENO5 at
  every face, plus four times the oracle's own spread under few-ulp perturbations of U (the
  derivative is set by rounding where smoothness indicators sit at WENO5's epsilon);
- stage outputs: stage states and cotangents to 1e-14 relative (the same operations, FP64
  atomics ordered differently); the dt-derivative identity to 1e-7 (central difference);
- reversal schedules: gradients to 1e-12 relative (same step VJPs, atomics order);
- windowed objective: adjoint against central differences to 1e-5 relative (h = 1e-4 for
  the scalings, 1e-3 degrees for the angle; FP64 forward runs); the angle gradient from the
  metric cotangents and from per-stage RHS differences within 1e-6 of each other (both
  difference the metrics over +- 1e-3 degrees, truncation ~1e-7)."""
import numpy as np
import pytest
import torch

from flame3d_mhd_gb300 import cases, ramp_adjoint
from flame3d_mhd_gb300.adjoint import gradient, trajectory_gradient
from flame3d_mhd_gb300.cases import params_copy
from flame3d_mhd_gb300.solver import Flame3D, side_stream
from oracle import oracle as orc
from test_gpu_adjoint import _kinetic_grad, smooth_generic_state

pytestmark = pytest.mark.gpu
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def _interior_random(shape, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(shape)
    a[I] = rng.standard_normal(a[I].shape)
    return a


@pytest.fixture(scope="module", params=["hybrid", "weno5"])
def ramp(request):
    """hybrid: the sensor's branches (UP7 near the smooth inflow); weno5: thresholds that leave
    it no choice, so the inflow profile's ghost cells feed WENO5 stencils too."""
    c = cases.compression_ramp(32, 16, 8, first_cell=1e-2, character=0)
    if request.param == "weno5":
        c["params"] = params_copy(c["params"], phi1=0.0, phi2=0.0, phi3=5.0)
    orc.set_inflow_profile(0, c["profile"])
    m, J, Q, U = orc.prepare(c["params"], c["Q"], c["x"], c["y"], c["z"])
    yield c, m, J, U
    orc.set_inflow_profile(0, None)
    orc.set_inflow_profile_tangent(0, None)


def _solver(c, m, J):
    s = Flame3D(c["params"])
    md, Jd = [dev(a) for a in m], dev(J)
    s.set_metrics(md, Jd)
    prof = dev(c["profile"])
    s.set_inflow_profile(0, prof)
    return s, (md, Jd, prof)


def _weno5_everywhere(P):
    return P.phi1 == 0.0 and P.phi2 == 0.0


def _rounding_spread(dot_of_U, U):
    """How far the oracle's own dot product moves when U is perturbed by a few ulps (relative
    1e-15). With WENO5 at every face, nearly uniform stencils (the free stream of the inflow)
    have smoothness indicators at its epsilon = 1e-16, where the weights' derivative scales as
    (V differences) / epsilon: the exact derivative is then set by rounding, and the oracle's
    moves by ~3e-8 of the sum of |terms| under such perturbations (the hybrid scheme, UP7 in
    that region: not at all)."""
    v0 = dot_of_U(U)
    return max(abs(dot_of_U(U * (1 + 1e-15 * np.random.default_rng(20 + k).uniform(-1, 1, U.shape))) - v0)
               for k in range(3))


def _profile_direction(prof, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(prof.shape) * np.abs(prof) * 1e-2


def test_rhs_profile_cotangent_dot_product(gpu_lib, ramp):
    c, m, J, U = ramp
    P = c["params"]
    s, keep = _solver(c, m, J)
    d = _profile_direction(c["profile"], 3)
    Lb = _interior_random(U.shape, 4)
    orc.set_inflow_profile_tangent(0, d)
    try:
        _, jvp = orc.rhs_jvp_u(P, U, np.zeros_like(U), m, J)
    finally:
        orc.set_inflow_profile_tangent(0, None)
    pb = torch.zeros_like(keep[2])
    s.set_inflow_profile_cotangent(0, pb)
    s.rhs_vjp(dev(U), dev(Lb))
    s.set_inflow_profile_cotangent(0, None)
    lhs = float((host(pb) * d).sum())
    rhs = float((Lb[I] * jvp[I]).sum())
    assert rhs != 0.0
    tol = 1e-10 * np.abs(Lb[I] * jvp[I]).sum()
    if _weno5_everywhere(P):
        def dot_of_U(Uv):
            orc.set_inflow_profile_tangent(0, d)
            try:
                return float((Lb[I] * orc.rhs_jvp_u(P, Uv, np.zeros_like(Uv), m, J)[1][I]).sum())
            finally:
                orc.set_inflow_profile_tangent(0, None)
        spread = _rounding_spread(dot_of_U, U)
        assert spread > 0.0
        tol += 4 * spread
    assert abs(lhs - rhs) <= tol, (lhs, rhs, tol)
    # once the buffer is unset nothing more is accumulated into it
    before = pb.clone()
    s.rhs_vjp(dev(U), dev(Lb))
    torch.cuda.synchronize()
    assert torch.equal(pb, before)
    s.close()


def test_rk3_steps_profile_cotangent_dot_product(gpu_lib, ramp):
    """Two chained step VJPs accumulate the profile cotangent of both steps."""
    c, m, J, U = ramp
    P = c["params"]
    s, keep = _solver(c, m, J)
    dt, steps = c["dt"], 2
    d = _profile_direction(c["profile"], 5)
    Ub = _interior_random(U.shape, 6)
    orc.set_inflow_profile_tangent(0, d)
    try:
        _, jvp = orc.rk3_jvp_u(P, steps, dt, U, np.zeros_like(U), m, J)
    finally:
        orc.set_inflow_profile_tangent(0, None)
    states = [dev(U)]
    Un, Qd = s.field(5), s.field(6)
    for _ in range(steps - 1):
        Ut = states[-1].clone()
        s.q_from_u(Ut, Qd)
        s.time_step(Ut, Un, Qd, dt, 1)
        states.append(Ut)
    pb = torch.zeros_like(keep[2])
    s.set_inflow_profile_cotangent(0, pb)
    g = dev(Ub)
    for Ut in reversed(states):
        g = s.rk3_step_vjp(dt, Ut, g)
    s.set_inflow_profile_cotangent(0, None)
    lhs = float((host(pb) * d).sum())
    rhs = float((Ub[I] * jvp[I]).sum())
    assert rhs != 0.0
    tol = 1e-10 * np.abs(Ub[I] * jvp[I]).sum()
    if _weno5_everywhere(P):
        def dot_of_U(Uv):
            orc.set_inflow_profile_tangent(0, d)
            try:
                return float((Ub[I] * orc.rk3_jvp_u(P, steps, dt, Uv, np.zeros_like(Uv), m, J)[1][I]).sum())
            finally:
                orc.set_inflow_profile_tangent(0, None)
        tol += 4 * _rounding_spread(dot_of_U, U)
    assert abs(lhs - rhs) <= tol, (lhs, rhs, tol)
    s.close()


def test_step_vjp_stage_outputs(gpu_lib, ramp):
    c, m, J, U = ramp
    s, keep = _solver(c, m, J)
    dt = c["dt"]
    Ud = dev(U)
    Ub = dev(_interior_random(U.shape, 7))
    plain = host(s.rk3_step_vjp(dt, Ud, Ub))
    Ust = torch.zeros((3, 5, *s.shape3), dtype=torch.float64, device="cuda")
    Lbt = torch.zeros_like(Ust)
    staged = host(s.rk3_step_vjp(dt, Ud, Ub, None, Ust, Lbt))
    scale = np.abs(plain[I]).max()
    assert np.abs(staged[I] - plain[I]).max() <= 1e-14 * scale
    # V_0 = U0, V_1 = U0 + dt L(U0); L_bar_2 = dt * 2/3 * Ubar_next
    assert torch.equal(Ust[0][I], Ud[I])
    L0 = s.rhs(s.q_from_u(Ud.clone()))
    assert float((Ust[1][I] - (Ud[I] + dt * L0[I])).abs().max()) <= 1e-14 * float(Ud[I].abs().max())
    assert float((Lbt[2][I] - dt * 2.0 / 3.0 * Ub[I]).abs().max()) <= 1e-14 * float((dt * Ub[I]).abs().max())
    # sum_s <L_bar_s, L(V_s)> = dt d/d(dt) <Ubar_next, U_1(dt)>
    acc = 0.0
    for k in range(3):
        Lk = s.rhs(s.q_from_u(Ust[k].clone()))
        acc += float((Lbt[k][I] * Lk[I]).sum())

    def step_dot(h):
        Ut, Un, Qd = Ud.clone(), s.field(5), s.field(6)
        s.q_from_u(Ut, Qd)
        s.time_step(Ut, Un, Qd, h, 1)
        return float((Ub[I] * Ut[I]).sum())
    e = 1e-3 * dt
    fd = dt * (step_dot(dt + e) - step_dot(dt - e)) / (2 * e)
    assert abs(fd - acc) <= 1e-7 * abs(acc), (fd, acc)
    s.close()


def test_bounded_reversal_matches_sqrt_checkpoints(gpu_lib):
    P, Q0, X, Y, Z, dt = smooth_generic_state(12)
    m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
    s = Flame3D(P)
    Jd = dev(J)
    s.set_metrics([dev(a) for a in m], Jd)
    N = 9
    with side_stream():
        _, g_ref = gradient(s, dev(U), dt, N, lambda UN: _kinetic_grad(UN, Jd), every=3)
        res = [trajectory_gradient(s, dev(U), dt, N, slots, final_grad=lambda UN: _kinetic_grad(UN, Jd))[1]
               for slots in (2, 3, 5, 10)]
    torch.cuda.synchronize()
    scale = float(g_ref[I].abs().max())
    for g in res:
        assert float((g[I] - g_ref[I]).abs().max()) <= 1e-12 * scale


def test_windowed_wall_force_gradient_vs_central_differences(gpu_lib):
    """J = dt * sum over the last 3 of 8 steps of the wall load (the wall-normal pressure
    force) on a 48x24x8 ramp; dJ/ds (24 inflow velocity scalings) along two seeded unit
    directions and dJ/dtheta against FP64 central differences, with 3 trajectory states held;
    the drag (x-force) gradient in theta likewise."""
    out = ramp_adjoint.main(["--nx", "48", "--ny", "24", "--nz", "8", "--first-cell", "1e-2", "--steps", "8",
                             "--window", "3", "--slots", "3", "--fd-dirs", "2", "--fd-h", "1e-4",
                             "--fd-angle-h", "1e-3", "--eta", "1e-3", "--mixed", "1"])
    assert out["reversal"]["recomputed_steps"] == out["reversal"]["planned_recomputed_steps"]
    for ch in out["checks"]:
        assert ch["adjoint"] != 0.0
        assert ch["rel_diff"] <= 1e-5, ch
    assert out["mixed_forward"]["J_rel_diff_vs_fp64"] <= 1e-5
    out = ramp_adjoint.main(["--nx", "48", "--ny", "24", "--nz", "8", "--first-cell", "1e-2", "--steps", "8",
                             "--window", "3", "--slots", "4", "--force", "x", "--fd-dirs", "0",
                             "--fd-angle-h", "1e-3", "--eta", "1e-3", "--mixed", "0"])
    (ch,) = out["checks"]
    assert ch["param"] == "theta_deg" and ch["rel_diff"] <= 1e-5, ch
    # the two ways to the angle gradient: metric cotangents, and per-stage RHS differences
    fd = ramp_adjoint.main(["--nx", "48", "--ny", "24", "--nz", "8", "--first-cell", "1e-2", "--steps", "8",
                            "--window", "3", "--slots", "4", "--force", "x", "--fd-dirs", "0", "--fd-angle-h", "",
                            "--eta", "1e-3", "--mixed", "0", "--angle-method", "fd"])
    g_adj, g_fd = out["gradient"]["dJdtheta_deg"], fd["gradient"]["dJdtheta_deg"]
    assert abs(g_adj - g_fd) <= 1e-6 * abs(g_fd), (g_adj, g_fd)


def test_lean_stage_cache_gives_the_same_step_vjp(gpu_lib, ramp):
    """adjoint_lean = 1 (one prepared stage state, re-prepared per stage) against the
    default three caches: the same VJP up to the order of FP64 atomics."""
    from flame3d_mhd_gb300.cases import params_copy
    c, m, J, U = ramp
    s, keep = _solver(c, m, J)
    cl = dict(c, params=params_copy(c["params"], adjoint_lean=1))
    sl, keepl = _solver(cl, m, J)
    Ud, Ub = dev(U), dev(_interior_random(U.shape, 9))
    g = host(s.rk3_step_vjp(c["dt"], Ud, Ub))
    gl = host(sl.rk3_step_vjp(c["dt"], Ud, Ub))
    assert np.abs(g[I] - gl[I]).max() <= 1e-14 * np.abs(g[I]).max()
    s.close()
    sl.close()

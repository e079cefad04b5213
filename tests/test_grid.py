"""Grid pipeline and the compression-ramp case on the CPU: the ghost-coordinate extension
against a literal per-cell restatement of SCU-benchmark/readfort.jl:34-95, the tanh
stretching, the ramp grid and inflow, and the oracle's inflow-profile ghost rule."""
import numpy as np
import pytest

from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import BC_INFLOW_PROFILE
from flame3d_mhd_gb300.grid import NG, compression_ramp_grid, extend_ghosts, tanh_beta
from oracle import oracle as orc


def _readfort_loops(x, y, z, solver=False):
    """readfort.jl:34-95 cell by cell, 1-based indices as in the Julia source, on arrays
    indexed [i, j, k] (Julia order); returns new arrays. solver=True: solver.jl:682-826 (one
    rank), which differs only in reflecting z across the eta faces (solver.jl:731-751)."""
    x, y, z = x.copy(), y.copy(), z.copy()
    Nxt, Nyt, Nzt = x.shape
    Nx, Ny, Nz = Nxt - 2 * NG, Nyt - 2 * NG, Nzt - 2 * NG
    A = lambda a, i, j, k: a[i - 1, j - 1, k - 1]

    def S(a, i, j, k, v):
        a[i - 1, j - 1, k - 1] = v

    for k in range(NG + 1, Nz + NG + 1):
        for j in range(NG + 1, Ny + NG + 1):
            for i in range(1, NG + 1):
                for a in (x, y, z):
                    S(a, i, j, k, 2 * A(a, NG + 1, j, k) - A(a, 2 * NG + 2 - i, j, k))
            for i in range(Nx + NG + 1, Nxt + 1):
                for a in (x, y, z):
                    S(a, i, j, k, 2 * A(a, Nx + NG, j, k) - A(a, 2 * NG + 2 * Nx - i, j, k))
        for i in range(NG + 1, Nx + NG + 1):
            for j in range(1, NG + 1):
                S(x, i, j, k, 2 * A(x, i, NG + 1, k) - A(x, i, 2 * NG + 2 - j, k))
                S(y, i, j, k, 2 * A(y, i, NG + 1, k) - A(y, i, 2 * NG + 2 - j, k))
                if solver:
                    S(z, i, j, k, 2 * A(z, i, NG + 1, k) - A(z, i, 2 * NG + 2 - j, k))
                else:
                    S(z, i, j, k, A(z, i, 2 * NG + 2 - j, k))
            for j in range(Ny + NG + 1, Nyt + 1):
                S(x, i, j, k, 2 * A(x, i, Ny + NG, k) - A(x, i, 2 * NG + 2 * Ny - j, k))
                S(y, i, j, k, 2 * A(y, i, Ny + NG, k) - A(y, i, 2 * NG + 2 * Ny - j, k))
                if solver:
                    S(z, i, j, k, 2 * A(z, i, Ny + NG, k) - A(z, i, 2 * NG + 2 * Ny - j, k))
                else:
                    S(z, i, j, k, A(z, i, 2 * NG + 2 * Ny - j, k))
        for jr, jb in ((range(Ny + NG + 1, Nyt + 1), Ny + NG), (range(1, NG + 1), NG + 1)):
            for ir, ib in ((range(1, NG + 1), NG + 1), (range(Nx + NG + 1, Nxt + 1), Nx + NG)):
                for j in jr:
                    for i in ir:
                        for a in (x, y, z):
                            S(a, i, j, k, A(a, i, jb, k) + A(a, ib, j, k) - A(a, ib, jb, k))
    for j in range(1, Nyt + 1):
        for i in range(1, Nxt + 1):
            for k in range(1, NG + 1):
                for a in (x, y, z):
                    S(a, i, j, k, 2 * A(a, i, j, NG + 1) - A(a, i, j, 2 * NG + 2 - k))
            for k in range(Nz + NG + 1, Nzt + 1):
                for a in (x, y, z):
                    S(a, i, j, k, 2 * A(a, i, j, Nz + NG) - A(a, i, j, 2 * NG + 2 * Nz - k))
    return x, y, z


@pytest.mark.parametrize("rule", ["readfort", "solver"])
def test_extend_ghosts_matches_readfort_loops(rule):
    rng = np.random.default_rng(3)
    shape = (6 + 2 * NG, 5 + 2 * NG, 7 + 2 * NG)  # (Nz+8, Ny+8, Nx+8)
    xyz = []
    for _ in range(3):
        a = np.zeros(shape)
        a[NG:-NG, NG:-NG, NG:-NG] = rng.standard_normal((6, 5, 7))
        xyz.append(a)
    got = extend_ghosts(*xyz, rule=rule)
    # the loops work on Julia-ordered [i, j, k] views
    ref = _readfort_loops(*[a.transpose(2, 1, 0) for a in xyz], solver=rule == "solver")
    for g, r in zip(got, ref):
        assert np.array_equal(g, r.transpose(2, 1, 0))


def test_tanh_beta_gives_the_first_cell():
    for n, h, first in ((256, 10.0, 1e-3), (32, 10.0, 1e-2), (64, 1.0, 1e-3)):
        b = tanh_beta(n, h, first)
        s1 = 1.0 - np.tanh(b * (1.0 - 1.0 / n)) / np.tanh(b)
        assert abs(h * s1 - first) <= 1e-9 * first
    with pytest.raises(ValueError):
        tanh_beta(10, 1.0, 0.2)  # larger than uniform spacing


def test_ramp_grid_is_body_fitted():
    x, y, z, beta = compression_ramp_grid(64, 32, 8, first_cell=1e-2)
    I = (slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    # the wall face (between the first ghost and the first cell rows) follows the ramp
    yw = 0.5 * (y[NG:-NG, NG - 1, NG:-NG] + y[NG:-NG, NG, NG:-NG])
    xs = x[NG, NG, NG:-NG]
    t = np.tan(np.radians(24.0))
    far = xs > 3.0
    assert np.allclose(yw[:, far], t * xs[far], atol=0.02)
    assert np.abs(yw[:, xs < -3.0]).max() < 0.02
    # grid lines increase monotonically in every direction
    assert (np.diff(x[I], axis=2) > 0).all() and (np.diff(y[I], axis=1) > 0).all() and (np.diff(z[I], axis=0) > 0).all()


def test_ramp_case_inflow_and_bcs():
    c = cases.compression_ramp(32, 24, 4, first_cell=1e-2)
    P, prof, w = c["params"], c["profile"], c["wall"]
    assert P.bc[0].kind == BC_INFLOW_PROFILE and prof.shape == (5, 4 + 2 * NG, 24 + 2 * NG)
    u = prof[1][NG, NG:-NG]
    assert (np.diff(u) >= 0).all() and abs(u[-1] - w["u_inf"]) < 1e-12 and u[0] < 0.6 * w["u_inf"]
    # Crocco-Busemann with the wall at the recovery temperature: T falls from T_w at the
    # wall to T_inf at the edge; mu(T_inf) = rho U delta / Re by the choice of C_s
    T = prof[4][NG, NG:-NG] / (prof[0][NG, NG:-NG] * P.rg)
    t_inf = (1.0 / 1.4) / 287.0
    assert (np.diff(T) <= 0).all() and T[0] <= w["t_w"] and T[-1] == pytest.approx(t_inf, rel=1e-12)
    assert P.c_s * t_inf ** 1.5 / (t_inf + P.t_s) == pytest.approx(2.9 / 1e5, rel=1e-12)


def test_oracle_inflow_profile_fill():
    c = cases.compression_ramp(16, 12, 4, first_cell=1e-2)
    P = c["params"]
    orc.set_inflow_profile(0, c["profile"])
    try:
        m, J, Q, U = orc.prepare(P, c["Q"], c["x"], c["y"], c["z"])
    finally:
        orc.set_inflow_profile(0, None)
    prof = c["profile"]
    # x- ghost cells at interior (j, k): the profile state; T = p / (rho Rg)
    for n, v in ((0, 0), (1, 1), (2, 2), (3, 3), (4, 4)):
        assert np.array_equal(Q[n, NG:-NG, NG:-NG, :NG], np.repeat(prof[v][NG:-NG, NG:-NG, None], NG, axis=2))
    assert np.array_equal(Q[5, NG:-NG, NG:-NG, 0], prof[4][NG:-NG, NG:-NG] / (prof[0][NG:-NG, NG:-NG] * P.rg))
    # corner (x-, y-): the isothermal wall mirrors the x- ghost column
    assert np.array_equal(Q[1, NG:-NG, NG - 1, :NG], -Q[1, NG:-NG, NG, :NG])
    # an unregistered profile poisons the ghosts instead of reading nothing
    Q2, U2 = Q.copy(), U.copy()
    orc.fill_ghosts(P, Q2, U2)
    assert np.isnan(Q2[0, NG:-NG, NG:-NG, :NG]).all()

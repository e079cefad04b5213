"""Python (ctypes) access to the CPU oracle liboracle_f3d.so.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline, never by the flame3d_mhd_gb300 package. All arrays are numpy float64 in the
reference layout, C-ordered (nvar, Nz+8, Ny+8, Nx+8). The library is built from
oracle/f3d_oracle.hpp by oracle/Makefile on first use.

Parity unpinned: the reference has no tests or golden vectors and cannot be run here (no
Julia); only its UP7 / CD6 coefficients are pinned, on its own Utils/FDMcoeffs.py.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_lib" / "liboracle_f3d.so"
NG = 4

_lib = None


def build(force: bool = False) -> Path:
    srcs = [HERE / "oracle_capi.cpp", HERE / "f3d_oracle.hpp", HERE / "f3d_numtypes.hpp",
            HERE.parent / "include" / "flame3d_gpu.h"]
    if force or not LIB.exists() or LIB.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.orc_set_threads.restype = C.c_int
        _lib.orc_set_threads.argtypes = [C.c_int]
        _lib.orc_set_inflow_profile.restype = None
        _lib.orc_set_inflow_profile.argtypes = [C.c_int, C.c_void_p]
        _lib.orc_set_inflow_profile_tangent.restype = None
        _lib.orc_set_inflow_profile_tangent.argtypes = [C.c_int, C.c_void_p]
        _lib.orc_set_coordinates.restype = None
        _lib.orc_set_coordinates.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    return _lib


_coords: list = []


def set_coordinates(x: np.ndarray | None, y: np.ndarray | None = None, z: np.ndarray | None = None) -> None:
    """Register the ghost-filled cell-centre coordinates the finite-volume schemes take
    their face geometry from (every later oracle call of such a scheme); None clears them."""
    if x is None:
        _coords.clear()
        lib().orc_set_coordinates(None, None, None)
        return
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z)]
    _coords[:] = arrs
    lib().orc_set_coordinates(*[a.ctypes.data for a in arrs])


def fvm_face_flux(P, d, eigen, phi, S, Q, U, x, y, z, with_branch=False):
    """FVM.jl face fluxes of direction d in the Fx/Fy/Fz shape."""
    F = np.zeros((5, *face_shape(P, d)))
    br = np.zeros(face_shape(P, d), dtype=np.int8) if with_branch else None
    xs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z)]
    lib().orc_fvm_face_flux(C.byref(P), C.c_int(d), C.c_int(int(eigen)), _p(phi), _p(S), _p(Q), _p(U),
                            _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(F), _p(br))
    return (F, br) if with_branch else F


def fvm_face_flux_ld(P, d, eigen, phi, S, Q, U, x, y, z):
    """fvm_face_flux evaluated in long double (the yardstick for FP64 rounding)."""
    F = np.zeros((5, *face_shape(P, d)))
    xs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z)]
    lib().orcld_fvm_face_flux(C.byref(P), C.c_int(d), C.c_int(int(eigen)), _p(phi), _p(S), _p(Q), _p(U),
                              _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(F))
    return F


_profiles: dict = {}


def set_inflow_profile(face: int, prof: np.ndarray | None) -> None:
    """Register the (5, Tb, Ta) state of an inflow-profile face for every oracle call
    (the layout of f3d_set_inflow_profile); None clears it."""
    if prof is None:
        _profiles.pop(face, None)
        lib().orc_set_inflow_profile(face, None)
        return
    a = np.ascontiguousarray(prof, dtype=np.float64)
    _profiles[face] = a  # keep it alive while registered
    lib().orc_set_inflow_profile(face, a.ctypes.data)


def set_inflow_profile_tangent(face: int, dprof: np.ndarray | None) -> None:
    """Register the tangent of an inflow profile (same layout) for the dual-number JVPs
    (rhs_jvp_u, rk3_jvp_u); None clears it."""
    if dprof is None:
        _profiles.pop(("d", face), None)
        lib().orc_set_inflow_profile_tangent(face, None)
        return
    a = np.ascontiguousarray(dprof, dtype=np.float64)
    _profiles[("d", face)] = a
    lib().orc_set_inflow_profile_tangent(face, a.ctypes.data)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(n)


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype in (np.float64, np.float32, np.int8) and a.flags.c_contiguous, "need C-contiguous arrays"
    return C.c_void_p(a.ctypes.data)


def _pp(arrs):
    return (C.c_void_p * len(arrs))(*[_p(a) for a in arrs])


def _dims(P):
    return (P.nz + 2 * NG, P.ny + 2 * NG, P.nx + 2 * NG)


def zeros(P, nvar: int = 1, dtype=np.float64) -> np.ndarray:
    s = _dims(P)
    return np.zeros(s if nvar == 1 else (nvar, *s), dtype=dtype)


def c2prim(P, U, Q=None):
    Q = zeros(P, 6) if Q is None else Q
    lib().orc_c2prim(C.byref(P), _p(U), _p(Q))
    return Q


def prim2c(P, Q, U=None):
    U = zeros(P, 5) if U is None else U
    lib().orc_prim2c(C.byref(P), _p(Q), _p(U))
    return U


def lincomb(P, U, Un, a, b):
    lib().orc_lincomb(C.byref(P), _p(U), _p(Un), C.c_double(a), C.c_double(b))


def fill_ghosts(P, Q, U):
    lib().orc_fill_ghosts(C.byref(P), _p(Q), _p(U))


def sensor(P, Q, phi=None):
    phi = zeros(P) if phi is None else phi
    lib().orc_sensor(C.byref(P), _p(Q), _p(phi))
    return phi


def metric_norm(P, a, b, c):
    s = zeros(P)
    lib().orc_metric_norm(C.byref(P), _p(a), _p(b), _p(c), _p(s))
    return s


def split(P, Q, A1, A2, A3, S):
    Fp, Fm = zeros(P, 5), zeros(P, 5)
    lib().orc_split(C.byref(P), _p(Q), _p(A1), _p(A2), _p(A3), _p(S), _p(Fp), _p(Fm))
    return Fp, Fm


def face_shape(P, d):
    n = [P.nz, P.ny, P.nx]
    n[2 - d] += 1
    return tuple(n)


def face_flux(P, d, phi, S, Fp, Fm, Q, A1, A2, A3, with_branch=False):
    F = np.zeros((5, *face_shape(P, d)))
    br = np.zeros(face_shape(P, d), dtype=np.int8) if with_branch else None
    lib().orc_face_flux(C.byref(P), C.c_int(d), _p(phi), _p(S), _p(Fp), _p(Fm), _p(Q), _p(A1), _p(A2), _p(A3),
                        _p(F), _p(br))
    return (F, br) if with_branch else F


def viscous(P, Q, m, J):
    s = (4, P.nz + 4, P.ny + 4, P.nx + 4)
    F = [np.zeros(s) for _ in range(3)]
    lib().orc_viscous(C.byref(P), _p(Q), _pp(m), _p(J), _p(F[0]), _p(F[1]), _p(F[2]))
    return F


def divergence(P, Fx, Fy, Fz, Fv, J, dt=0.0, U=None):
    """U += dt J (dF + dFv) when U is given (div.jl), else returns dUdt."""
    fv = Fv if Fv is not None else [None, None, None]
    out = None if U is not None else zeros(P, 5)
    lib().orc_divergence(C.byref(P), _p(Fx), _p(Fy), _p(Fz), _p(fv[0]), _p(fv[1]), _p(fv[2]), _p(J),
                         C.c_double(dt), _p(U), _p(out))
    return out


def metrics(P, x, y, z):
    m = [zeros(P) for _ in range(9)]
    J = zeros(P)
    lib().orc_metrics(C.byref(P), _p(x), _p(y), _p(z), _pp(m), _p(J))
    return m, J


def rhs(P, Q, m, J, with_branches=False):
    out = zeros(P, 5)
    nb = sum(int(np.prod(face_shape(P, d))) for d in range(3))
    br = np.zeros(nb, dtype=np.int8) if with_branches else None
    lib().orc_rhs(C.byref(P), _p(Q), _pp(m), _p(J), _p(out), _p(br))
    if not with_branches:
        return out
    parts, off = [], 0
    for d in range(3):
        n = int(np.prod(face_shape(P, d)))
        parts.append(br[off:off + n].reshape(face_shape(P, d)))
        off += n
    return out, parts


def rhs_ld(P, Q, m, J):
    """(dUdt, flux_scale[5]) in extended precision; flux_scale is the per-variable max of
    J * sum |face fluxes| the RHS differences (the conditioning yardstick)."""
    out = zeros(P, 5)
    scale = np.zeros(5)
    lib().orcld_rhs(C.byref(P), _p(Q), _pp(m), _p(J), _p(out), _p(scale))
    return out, scale


def local_dt(P, Q, m, J):
    """compute_dt (utils.jl:73-99) at interior cells (ghost cells 0)."""
    dt = zeros(P)
    lib().orc_local_dt(C.byref(P), _p(Q), _pp(m), _p(J), _p(dt))
    return dt


def filter_pass(P, U, Un, Q):
    """One pass of params.filter over U in place (three directions, Un the per-direction copy)."""
    lib().orc_filter(C.byref(P), _p(U), _p(Un), _p(Q))


def rk3_ld(P, nsteps, dt, U, Un, Q, m, J):
    """nsteps SSP-RK3 steps in extended precision (in place, rounded back to FP64)."""
    lib().orcld_rk3(C.byref(P), C.c_int(nsteps), C.c_double(dt), _p(U), _p(Un), _p(Q), _pp(m), _p(J))


def rk3(P, nsteps, dt, U, Un, Q, m, J):
    lib().orc_rk3(C.byref(P), C.c_int(nsteps), C.c_double(dt), _p(U), _p(Un), _p(Q), _pp(m), _p(J))


class PersistentSolver:
    """Oracle workspace kept across calls (for timing the CPU baseline)."""

    def __init__(self, P, m, J):
        self.P, self._keep = P, (m, J)
        l = lib()
        l.orc_solver_create.restype = C.c_void_p
        l.orc_solver_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.orc_solver_rk3.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        l.orc_solver_destroy.argtypes = [C.c_void_p]
        self._marr = _pp(m)
        self.h = l.orc_solver_create(C.addressof(P), C.addressof(self._marr), _p(J))

    def rk3(self, nsteps, dt, U, Un, Q):
        lib().orc_solver_rk3(self.h, nsteps, dt, _p(U), _p(Un), _p(Q))

    def close(self):
        if self.h:
            lib().orc_solver_destroy(self.h)
            self.h = None


def rk3_stage(P, stage, dt, U, Un, Q, m, J):
    lib().orc_rk3_stage(C.byref(P), C.c_int(stage), C.c_double(dt), _p(U), _p(Un), _p(Q), _pp(m), _p(J))


def rhs32(P, Q32, m32, J32):
    out = zeros(P, 5, np.float32)
    lib().orc32_rhs(C.byref(P), _p(Q32), _pp(m32), _p(J32), _p(out))
    return out


def c2prim32(P, U32):
    """c2Prim in the reference's Float32 arithmetic (interior cells; the rest of Q zero)."""
    Q = zeros(P, 6, np.float32)
    lib().orc32_c2prim(C.byref(P), _p(U32), _p(Q))
    return Q


def prim2c32(P, Q32):
    U = zeros(P, 5, np.float32)
    lib().orc32_prim2c(C.byref(P), _p(Q32), _p(U))
    return U


def fill_ghosts32(P, Q32, U32):
    lib().orc32_fill_ghosts(C.byref(P), _p(Q32), _p(U32))


def rk3_32(P, nsteps, dt, U, Un, Q, m, J):
    lib().orc32_rk3(C.byref(P), C.c_int(nsteps), C.c_float(dt), _p(U), _p(Un), _p(Q), _pp(m), _p(J))


def rhs_jvp_m(P, Q, m, dm, J, dJ):
    """(dUdt, d dUdt) of the RHS at fixed Q along the metric tangents (dm, dJ), forward mode."""
    r, dr = zeros(P, 5), zeros(P, 5)
    lib().orc_rhs_jvp_m(C.byref(P), _p(Q), _pp(m), _pp(dm), _p(J), _p(dJ), _p(r), _p(dr))
    return r, dr


def rk3_jvp_m(P, nsteps, dt, U0, m, dm, J, dJ):
    u, du = zeros(P, 5), zeros(P, 5)
    lib().orc_rk3_jvp_m(C.byref(P), C.c_int(nsteps), C.c_double(dt), _p(U0), _pp(m), _pp(dm), _p(J), _p(dJ),
                        _p(u), _p(du))
    return u, du


def rhs_jvp_u(P, U, dU, m, J):
    """(dUdt, d dUdt) of U -> c2Prim -> ghost fill -> RHS, forward mode."""
    r, dr = zeros(P, 5), zeros(P, 5)
    lib().orc_rhs_jvp_u(C.byref(P), _p(U), _p(dU), _pp(m), _p(J), _p(r), _p(dr))
    return r, dr


def rk3_jvp_u(P, nsteps, dt, U0, dU0, m, J):
    u, du = zeros(P, 5), zeros(P, 5)
    lib().orc_rk3_jvp_u(C.byref(P), C.c_int(nsteps), C.c_double(dt), _p(U0), _p(dU0), _pp(m), _p(J), _p(u), _p(du))
    return u, du


def rhs_opcount(P, Q, m, J) -> dict:
    out = np.zeros(5)
    lib().orc_rhs_opcount(C.byref(P), _p(Q), _pp(m), _p(J), _p(out))
    return dict(add=out[0], mul=out[1], div=out[2], sqrt=out[3], cmp=out[4])


def prepare(P, case_Q, x, y, z):
    """Metrics from coordinates, U = prim2c(Q) and the ghost fill, as solver.jl:238-345."""
    m, J = metrics(P, x, y, z)
    Q = np.ascontiguousarray(case_Q, dtype=np.float64).copy()
    U = prim2c(P, Q)
    fill_ghosts(P, Q, U)
    return m, J, Q, U

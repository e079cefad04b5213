"""Runtime for the reference's Julia kernels translated by jl2py.py (test infrastructure).

The translated kernels keep the reference's statements; this module gives them what CUDA.jl
and run.jl gave them:
- arrays taking Julia's 1-based, column-major subscripts A[i, j, k, n] over this
  repository's [n, k, j, i] layout (JArray);
- the thread index of a launch (one thread at a time: blockIdx = blockDim = 1,
  threadIdx = (i, j, k)) and Julia's max / min (a NaN wins), sqrt (NaN below 0), ifelse,
  zero, eps(Float32);
- the global constants of run.jl:4-13, 57-77 (LES_smag, LES_wale, γ, Rg, Cp, C_s, T_s, Pr, Ncons,
  the hybrid thresholds, Linear, NG, Nxp, Nyp, Nzp) from an f3d_params;
- the launch sequence of one RHS: the sensor (solver.jl:424), the split and the
  reconstruction of each direction (solver.jl:133-188) or, for the finite-volume schemes, the
  face kernels of FVM.jl (solver.jl:21-31), the viscous fluxes and div (solver.jl:429) into a
  zero accumulator with dt = 1, so it ends holding J times the flux divergence, the RHS;
- prim2c, c2Prim and the ghost fill of one process for boundary.jl's own boundary set, the
  RK3 stage loop of time_step, its local time step and its filtering pass;
- the metrics and J of parse_mesh.jl and of SCU-benchmark/readfort.jl (scripts, each
  translated as the body of one function), and the ghost coordinates of readfort.jl's
  generateXYZ and of solver.jl's extrapolation.

Every value is a binary64 NumPy scalar (IEEE: 0/0 is NaN, as in Julia): the reference's
algorithm in FP64, in its own operation order. With typed=True (a module translated with
Julia's types) the arrays are Float32, run.jl's constants Float32 and the helpers keep and
promote types as Julia does: the reference's own precision. Slow (one Python call per
thread): grids of a few hundred cells.
"""
from __future__ import annotations

import math
import unicodedata
from pathlib import Path
from types import SimpleNamespace

import numpy as np

NG = 4


class _Range:
    """Julia's a:b in a subscript (inclusive, 1-based)."""

    __slots__ = ("lo", "hi")

    def __init__(self, lo, hi):
        self.lo, self.hi = lo, hi


_ALL = _Range(None, None)


def _py_index(x):
    if isinstance(x, _Range):
        return slice(None if x.lo is None else x.lo - 1, x.hi)
    return x - 1


class JArray:
    """A[i, j, k, n] (1-based, Julia's order) over a numpy array stored [n, k, j, i]; a:b and :
    subscripts give JArray views; arithmetic on whole arrays is elementwise (Julia's @.)."""

    __slots__ = ("a",)

    def __init__(self, a: np.ndarray):
        self.a = a

    def _key(self, idx):
        idx = idx if isinstance(idx, tuple) else (idx,)
        return tuple(_py_index(x) for x in reversed(idx)), any(isinstance(x, _Range) for x in idx)

    def __getitem__(self, idx):
        key, sliced = self._key(idx)
        return JArray(self.a[key]) if sliced else self.a[key]  # a NumPy scalar: IEEE 0/0 = NaN, as Julia

    def __setitem__(self, idx, v):
        key, _ = self._key(idx)
        self.a[key] = v.a if isinstance(v, JArray) else v

    def _fill(self, v):
        self.a[...] = v

    # elementwise arithmetic (the fused broadcasts of @. evaluate the same operations per element)
    def _o(self, x):
        return x.a if isinstance(x, JArray) else x

    def __add__(self, x): return self.a + self._o(x)
    def __radd__(self, x): return self._o(x) + self.a
    def __sub__(self, x): return self.a - self._o(x)
    def __rsub__(self, x): return self._o(x) - self.a
    def __mul__(self, x): return self.a * self._o(x)
    def __rmul__(self, x): return self._o(x) * self.a
    def __truediv__(self, x): return self.a / self._o(x)
    def __rtruediv__(self, x): return self._o(x) / self.a
    def __neg__(self): return -self.a


def _bset(lhs, v):
    lhs.a[...] = v.a if isinstance(v, JArray) else v


_thread = SimpleNamespace(x=1, y=1, z=1)
_one = SimpleNamespace(x=1, y=1, z=1)


def _jmax(*v):
    for x in v:
        if x != x:
            return x
    return max(v)


def _jmin(*v):
    for x in v:
        if x != x:
            return x
    return min(v)


def _sqrt(x):
    return np.float64(math.sqrt(x)) if x >= 0 else np.float64("nan")


def _mat(r, c=None):
    return JArray(np.zeros(r if c is None else (c, r)))


def _tjmax(*v):
    """Julia's max on typed values: NaN wins, the result in the promoted type."""
    for x in v:
        if x != x:
            return np.result_type(*v).type(x)
    return np.result_type(*v).type(max(v))


def _tjmin(*v):
    for x in v:
        if x != x:
            return np.result_type(*v).type(x)
    return np.result_type(*v).type(min(v))


def _tsqrt(x):
    """sqrt in the argument's precision (an Int gives Float64); NaN below 0, as on the GPU."""
    return np.sqrt(x if isinstance(x, np.floating) else np.float64(x))


def _tmat(r, c=None, bits=64):
    return JArray(np.zeros(r if c is None else (c, r), dtype=np.float32 if bits == 32 else np.float64))


def _sinh(x):
    """sinh in binary64, rounded to the argument's type (for Float32: Julia's own Float32 sinh
    may differ from this in the last bit)."""
    r = np.float64(math.sinh(float(x)))
    return r.astype(x.dtype) if isinstance(x, np.floating) else r


HELPERS = dict(
    blockIdx=lambda: _one, blockDim=lambda: _one, threadIdx=lambda: _thread, sinh=_sinh,
    max=_jmax, min=_jmin, sqrt=_sqrt, abs=abs,
    ifelse=lambda c, a, b: a if c else b, zero=lambda a: 0.0,
    _eps32=lambda: 2.0 ** -23, _mat=_mat, _f32=float, _f64=float,
    _p2=lambda x: x * x, _p3=lambda x: x * x * x,  # Julia's literal powers (Base.literal_pow)
    _r=_Range, _all=_ALL, _bset=_bset, _vec=lambda *v: JArray(np.array(v, dtype=np.float64)),
    _zeros=lambda *dims: JArray(np.zeros(tuple(reversed(dims)))),
)


def kernels(module_path: Path | str, P, typed: bool = False) -> dict:
    """The translated kernels with the run.jl constants of the parameter set P. typed: for a
    module translated with Julia's types (jl2py typed), the constants in run.jl's types
    (Float32, computed in Float32 where run.jl computes them) and type-preserving helpers."""
    g = dict(HELPERS)
    f = np.float32 if typed else float
    gamma, rg = f(P.gamma), f(P.rg)
    up7 = [-3 / 420, 25 / 420, -101 / 420, 319 / 420, 214 / 420, -38 / 420, 4 / 420]
    cd6 = [0.0, 1 / 60, -2 / 15, 37 / 60, 37 / 60, -2 / 15, 1 / 60]
    lp = f(P.linear_phi)
    if typed:  # SVector{7, Float32}(Float64 quotients); Linear = UP7 * Linear_ϕ + CD6 * (1 - Linear_ϕ)
        linear = (np.array(up7).astype(np.float32) * lp + np.array(cd6).astype(np.float32) * (np.float32(1) - lp))
        g.update(_f32=np.float32, _f64=np.float64, _eps32=lambda: np.float32(2.0 ** -23), _mat=_tmat,
                 _zerosT=lambda bits, *dims: JArray(np.zeros(tuple(reversed(dims)),
                                                             np.float32 if bits == 32 else np.float64)),
                 max=_tjmax, min=_tjmin, sqrt=_tsqrt, zero=lambda a: type(a)(0) if isinstance(a, np.generic) else 0)
    else:
        linear = np.array([u * lp + c * (1.0 - lp) for u, c in zip(up7, cd6)])
    g.update({
        "γ": gamma, "Rg": rg, "Cp": f(P.cp) if P.cp else rg * gamma / (gamma - 1),
        "C_s": f(P.c_s), "T_s": f(P.t_s), "Pr": f(P.pr),
        "Ncons": 5, "Nprim": 6, "NG": NG, "Nxp": int(P.nx), "Nyp": int(P.ny), "Nzp": int(P.nz),
        "hybrid_ϕ1": f(P.phi1), "hybrid_ϕ2": f(P.phi2), "hybrid_ϕ3": f(P.phi3),
        "Linear": JArray(linear),
        "LES_smag": int(getattr(P, "les", 0)) == 1, "LES_wale": int(getattr(P, "les", 0)) == 2,
        "Nx": int(P.nx), "Ny": int(P.ny), "Nz": int(P.nz),
        "Nx_tot": int(P.nx) + 2 * NG, "Ny_tot": int(P.ny) + 2 * NG, "Nz_tot": int(P.nz) + 2 * NG,
    })
    # Python reads identifiers NFKC-normalised (the ϕ of hybrid_ϕ1 becomes φ): so must the names
    g = {unicodedata.normalize("NFKC", name): v for name, v in g.items()}
    ext = (int(P.nx) + 2 * NG, int(P.ny) + 2 * NG, int(P.nz) + 2 * NG)
    g["_cuda"] = lambda fn, *args: launch(fn, ext, *args)  # the grid of every @cuda launch
    g["Nprocs"] = JArray(np.array([1, 1, 1]))
    exec(compile(Path(module_path).read_text(), str(module_path), "exec"), g)
    return g


def launch(fn, ext, *args):
    """Every thread (i, j, k) of a grid covering ext = (X, Y, Z), one after the other (IEEE
    exceptions quiet: a division by zero gives inf or NaN, as on the GPU)."""
    X, Y, Z = ext
    with np.errstate(all="ignore"):
        for k in range(1, Z + 1):
            for j in range(1, Y + 1):
                for i in range(1, X + 1):
                    _thread.x, _thread.y, _thread.z = i, j, k
                    fn(*args)


def is_reference_bcs(P) -> bool:
    """The boundary set boundary.jl hard-codes: x- the free stream (rho 1, u 0.5, p 1/1.4),
    x+ zero gradient, y- an adiabatic no-slip wall, y+ the free stream, z periodic."""
    k = [int(b.kind) for b in P.bc]
    fs = [P.bc[0], P.bc[3]]
    return k == [1, 2, 3, 1, 0, 0] and all(
        (float(b.rho), float(b.u), float(b.v), float(b.w), float(b.p)) == (1.0, 0.5, 0.0, 0.0, 1.0 / 1.4) for b in fs)


def state_and_ghosts(module_path, P, Q: np.ndarray, typed: bool = False):
    """U = prim2c(Q) at every cell (utils.jl:33-54); then, as a stage does
    (solver.jl:438-443), Q = c2Prim(U) at the interior (utils.jl:2-30) and the ghost fill of one
    process (boundary.jl's fillGhost: fill_x, fill_y, fill_z; the periodic exchange of mpi.jl on
    one process only copies layers that fill_y and fill_z overwrite afterwards). Returns
    (U from prim2c, Q after c2Prim and the fill, U after the fill). typed: Float32 arrays and a
    module translated with Julia's types."""
    if not is_reference_bcs(P):
        raise ValueError("boundary.jl hard-codes one boundary set; these parameters have another")
    k = kernels(module_path, P, typed)
    dtype = np.float32 if typed else np.float64
    nx, ny, nz = int(P.nx), int(P.ny), int(P.nz)
    ext = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    U = JArray(np.zeros((5, *Q.shape[1:]), dtype))
    launch(k["prim2c"], ext, U, JArray(Q.astype(dtype)))
    U0 = U.a.copy()
    Q2 = JArray(np.zeros(Q.shape, dtype))
    launch(k["c2Prim"], ext, U, Q2)
    k["fillGhost"](Q2, U, 0, 0)  # rank (0, 0) of one process
    return U0, Q2.a, U.a


def _advance(k, P, Qj, m, S, Jj, U, dt, xyz=None, Ustate=None, lts_dt=None):
    """The sensor, flowAdvance (solver.jl:19-188) and div (U += dt J (...)). Finite-difference
    schemes: split and reconstruction per direction. Finite-volume schemes (P.scheme 1:
    Eigen_reconstruct_*, 2: Conser_reconstruct_*): the face kernels of solver.jl:21-31 on the
    cell-centre coordinates xyz, reading Ustate (default U, the stage's state, which div then
    updates, as in the reference). lts_dt: the per-cell time steps of compute_dt, applied by
    div_LTS (solver.jl:425-426) in place of div with the global dt."""
    nx, ny, nz = int(P.nx), int(P.ny), int(P.nz)
    ext = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    shape, dt_ = Qj.a.shape[1:], Qj.a.dtype  # intermediates in the state's element type
    phi = JArray(np.zeros(shape, dt_))
    launch(k["shockSensor"], ext, phi, Qj)
    F = [JArray(np.zeros((5, nz, ny, nx + 1), dt_)), JArray(np.zeros((5, nz, ny + 1, nx), dt_)),
         JArray(np.zeros((5, nz + 1, ny, nx), dt_))]
    scheme = int(getattr(P, "scheme", 0))
    if scheme:
        name = "Eigen_reconstruct_" if scheme == 1 else "Conser_reconstruct_"
        for d, suf in enumerate("ijk"):
            launch(k[name + suf], ext, Qj, U if Ustate is None else Ustate, phi, S[d], F[d], *xyz)
    else:
        Fp, Fm = JArray(np.zeros((5, *shape), dt_)), JArray(np.zeros((5, *shape), dt_))
        split = k[SPLITS[int(P.split_method)]]
        for d, name in enumerate("xyz"):
            launch(split, ext, Qj, Fp, Fm, S[d], m[3 * d], m[3 * d + 1], m[3 * d + 2])
            if int(P.character):
                launch(k["advect_" + name + "c"], ext, F[d], phi, S[d], Fp, Fm, Qj, m[3 * d], m[3 * d + 1], m[3 * d + 2])
            else:
                launch(k["advect_" + name], ext, F[d], phi, S[d], Fp, Fm, 5)
    Fv = [JArray(np.zeros((4, nz + 4, ny + 4, nx + 4), dt_)) for _ in range(3)]
    if int(P.viscous):
        launch(k["viscousFlux"], ext, *Fv, Qj, *m, Jj)
    if lts_dt is None:
        launch(k["div"], (nx, ny, nz), U, *F, *Fv, dt, Jj)
    else:
        launch(k["div_LTS"], (nx, ny, nz), U, *F, *Fv, lts_dt, Jj)


def _coords(P, xyz):
    if int(getattr(P, "scheme", 0)) == 0:
        return None
    if xyz is None:
        raise ValueError("the finite-volume schemes need the cell-centre coordinates")
    return [JArray(np.asarray(a, dtype=np.float64)) for a in xyz]


def _metric_arrays(metrics, J, dtype=np.float64):
    m = [JArray(metrics[n].astype(dtype)) for n in range(9)]
    # solver.jl:286-288: s = sqrt(a^2 + b^2 + c^2) of each metric row, in the arrays' type
    S = [JArray(np.sqrt(m[3 * d].a ** 2 + m[3 * d + 1].a ** 2 + m[3 * d + 2].a ** 2)) for d in range(3)]
    return m, S, JArray(J.astype(dtype))


def rk3_steps(module_path, P, U0: np.ndarray, metrics, J, dt: float, nsteps: int, Q0: np.ndarray | None = None,
              xyz=None, typed: bool = False):
    """nsteps SSP-RK3 steps of time_step's loop (solver.jl:410-470) from the conserved state U0
    and its ghost-filled primitive state Q0 (formed from U0 as a stage forms it when not
    given), for boundary.jl's boundary set: with P.lts, compute_dt before the first stage of
    each step and div_LTS in every stage; with P.filter, after every P.filter_interval-th step
    the filtering pass of solver.jl:446-470 (step counter from 1); xyz: the cell-centre
    coordinates (x, y, z) for the finite-volume schemes; typed: Float32 arrays, dt and linComb
    weights (0.25f0, 0.75f0, 2/3f0, 1/3f0) and a module translated with Julia's types.
    Returns (U, Q)."""
    if not is_reference_bcs(P):
        raise ValueError("boundary.jl hard-codes one boundary set; these parameters have another")
    k = kernels(module_path, P, typed)
    dtype = np.float32 if typed else np.float64
    f = np.float32 if typed else float
    nx, ny, nz = int(P.nx), int(P.ny), int(P.nz)
    ext = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    m, S, Jj = _metric_arrays(metrics, J, dtype)
    xyz = _coords(P, xyz)
    U = JArray(U0.astype(dtype).copy())
    dt = f(dt)
    if Q0 is None:
        Q = JArray(np.zeros((6, *U0.shape[1:]), dtype))
        launch(k["c2Prim"], ext, U, Q)
        k["fillGhost"](Q, U, 0, 0)
    else:
        Q = JArray(Q0.astype(dtype).copy())
    lts = bool(int(P.lts))
    if lts:
        k["LTS_CFL"] = f(P.lts_cfl)
        lts_dt = JArray(np.zeros(U0.shape[1:], dtype))
    for tt in range(1, nsteps + 1):
        for krk in (1, 2, 3):
            if krk == 1:
                Un = JArray(U.a.copy())
                if lts:
                    launch(k["compute_dt"], ext, lts_dt, Q, Jj, *S)
            _advance(k, P, Q, m, S, Jj, U, dt, xyz, lts_dt=lts_dt if lts else None)
            if krk == 2:
                launch(k["linComb"], ext, U, Un, 5, f(0.25), f(0.75))
            elif krk == 3:
                launch(k["linComb"], ext, U, Un, 5, f(2) / f(3), f(1) / f(3))
            launch(k["c2Prim"], ext, U, Q)
            k["fillGhost"](Q, U, 0, 0)
        if int(P.filter) and tt % int(P.filter_interval) == 0:
            _filter(k, P, U, Q, f)
    return U.a, Q.a


def metrics(module_path, P, x: np.ndarray, y: np.ndarray, z: np.ndarray, typed: bool = False,
            source: str = "parse_mesh"):
    """parse_mesh.jl:139-248 (source "readfort": SCU-benchmark/readfort.jl:104-208) on the
    coordinates with ghosts: the nine J^-1-scaled metrics (dξ/dx, dξ/dy, dξ/dz, dη/dx, ...,
    dζ/dz) and J, each (Nz_tot, Ny_tot, Nx_tot). typed: the script's own precision (Float32
    coordinates and arrays; parse_mesh.jl's Float64 coefficients, readfort.jl's Float32 ones)
    from a module translated with Julia's types."""
    k = kernels(module_path, P, typed)
    dtype = np.float32 if typed else np.float64
    fn = k["_metrics" if source == "parse_mesh" else "_metrics_readfort"]
    m, J = fn(*(JArray(np.asarray(c, dtype=dtype)) for c in (x, y, z)))
    return np.stack([a.a for a in m]), J.a


def ghost_coordinates(module_path, P, x: np.ndarray, y: np.ndarray, z: np.ndarray, rule: str = "readfort",
                      typed: bool = False):
    """Ghost cell-centre coordinates from coordinates with the interior filled ((Nz_tot,
    Ny_tot, Nx_tot) each): rule "readfort" runs SCU-benchmark/readfort.jl:34-99 (the
    reflections and edge completions of generateXYZ, then ./= 1000), rule "solver" runs
    solver.jl's extrapolation on one rank. typed: Float32 arrays (the reference's) and a
    module translated with Julia's types."""
    k = kernels(module_path, P, typed)
    dtype = np.float32 if typed else np.float64
    X, Y, Z = (JArray(np.array(a, dtype=dtype, copy=True)) for a in (x, y, z))
    if rule == "readfort":
        k["_ghosts_readfort"](X, Y, Z)
    else:
        k["extrapolation"](X, Y, Z, 0, 0, 0)
    return X.a, Y.a, Z.a


def flat_plate(module_path, P, lx=2.0, ly=0.1, lz=0.1, factor=3.5, typed: bool = False):
    """parse_mesh.jl's flat-plate coordinates (:38-136) for the grid of P: every cell mapped
    (x = Lx xi, y = stretching_y(eta), z = Lz zeta), then the ghost layers reflected; its
    Float32 constants Lx, Ly, Lz, stretch_factor_y from the arguments."""
    k = kernels(module_path, P, typed)
    f, dtype = (np.float32, np.float32) if typed else (float, np.float64)
    shape = (int(P.nz) + 2 * NG, int(P.ny) + 2 * NG, int(P.nx) + 2 * NG)
    X, Y, Z = (JArray(np.zeros(shape, dtype)) for _ in range(3))
    k["_flat_plate"](X, Y, Z, f(lx), f(ly), f(lz), f(factor))
    return X.a, Y.a, Z.a


def fvm_faces(module_path, P, Q: np.ndarray, metrics: np.ndarray, xyz):
    """The finite-volume face fluxes of the three directions, each in the Fx / Fy / Fz shape,
    as flowAdvance's finite-volume branch launches them (solver.jl:21-31): Eigen_reconstruct_*
    (P.scheme 1) or Conser_reconstruct_* (2) of FVM.jl on the ghost-filled primitive state Q,
    U = prim2c(Q) at every cell, the reference's sensor, the metric-row norms s1, s2, s3 and
    the cell-centre coordinates xyz = (x, y, z)."""
    k = kernels(module_path, P)
    nx, ny, nz = int(P.nx), int(P.ny), int(P.nz)
    ext = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    _, S, _ = _metric_arrays(metrics, np.zeros(1))
    Qj = JArray(Q.astype(np.float64))
    U, phi = JArray(np.zeros((5, *Q.shape[1:]))), JArray(np.zeros(Q.shape[1:]))
    launch(k["prim2c"], ext, U, Qj)
    launch(k["shockSensor"], ext, phi, Qj)
    F = [JArray(np.zeros((5, nz, ny, nx + 1))), JArray(np.zeros((5, nz, ny + 1, nx))),
         JArray(np.zeros((5, nz + 1, ny, nx)))]
    name = "Eigen_reconstruct_" if int(P.scheme) == 1 else "Conser_reconstruct_"
    for d, suf in enumerate("ijk"):
        launch(k[name + suf], ext, Qj, U, phi, S[d], F[d], *_coords(P, xyz))
    return [f.a for f in F]


def prim2c(module_path, P, Q: np.ndarray) -> np.ndarray:
    """prim2c (utils.jl:33-54) at every cell."""
    k = kernels(module_path, P)
    U = JArray(np.zeros((5, *Q.shape[1:])))
    launch(k["prim2c"], (int(P.nx) + 2 * NG, int(P.ny) + 2 * NG, int(P.nz) + 2 * NG), U, JArray(Q.astype(np.float64)))
    return U.a


def local_dt(module_path, P, Q: np.ndarray, metrics, J) -> np.ndarray:
    """compute_dt (utils.jl:73-99) with LTS_CFL = P.lts_cfl: the per-cell time step at the
    interior (zero elsewhere)."""
    k = kernels(module_path, P)
    k["LTS_CFL"] = float(P.lts_cfl)
    m, S, Jj = _metric_arrays(metrics, J)
    dt = JArray(np.zeros(Q.shape[1:]))
    ext = (int(P.nx) + 2 * NG, int(P.ny) + 2 * NG, int(P.nz) + 2 * NG)
    launch(k["compute_dt"], ext, dt, JArray(Q.astype(np.float64)), Jj, *S)
    return dt.a


def _filter(k, P, Uj, Qj, f=float):
    """The filtering pass of time_step (solver.jl:446-470) over Uj in place: per direction,
    Un = U, then the pressure sensor pre_d and the shock-capturing filter_d (P.filter 2) or the
    linear linearFilter_d (P.filter 1) with filtering_s0 = P.filter_s0, filtering_rth =
    P.filter_rth."""
    ext = (int(P.nx) + 2 * NG, int(P.ny) + 2 * NG, int(P.nz) + 2 * NG)
    sc = JArray(np.zeros(Qj.a.shape[1:], Qj.a.dtype))
    s0, rth = f(P.filter_s0), f(P.filter_rth)
    for d in "xyz":
        Un = JArray(Uj.a.copy())
        if int(P.filter) == 2:
            launch(k["pre_" + d], ext, Qj, sc, rth)
            launch(k["filter_" + d], ext, Uj, Un, sc, s0)
        else:
            launch(k["linearFilter_" + d], ext, Uj, Un, s0)


def filter_pass(module_path, P, U: np.ndarray, Q: np.ndarray) -> np.ndarray:
    """One filtering pass of time_step (solver.jl:446-470) over a copy of U (_filter)."""
    Uj, Qj = JArray(U.astype(np.float64).copy()), JArray(Q.astype(np.float64))
    _filter(kernels(module_path, P), P, Uj, Qj)
    return Uj.a


SPLITS = ("fluxSplit_SW", "fluxSplit_LF", "fluxSplit_VL", "fluxSplit_AUSM")


def rhs(module_path, P, Q: np.ndarray, metrics: np.ndarray, J: np.ndarray, xyz=None, typed: bool = False) -> np.ndarray:
    """dU/dt at the interior (zero elsewhere) of the reference's RHS from the ghost-filled
    primitive state Q (6, Nt...), the nine J^-1-scaled metrics and J: the advance of one stage
    into a zero accumulator with dt = 1. The finite-volume schemes reconstruct U = prim2c(Q)
    (utils.jl:33-54, every cell) on the cell-centre coordinates xyz = (x, y, z). typed: a module
    translated with Julia's types, on Float32 arrays (the reference's CuArray{Float32})."""
    k = kernels(module_path, P, typed)
    dtype = np.float32 if typed else np.float64
    m, S, Jj = _metric_arrays(metrics, J, dtype)
    Qj = JArray(Q.astype(dtype))
    xyz = _coords(P, xyz)
    Ustate = None
    if xyz is not None:
        Ustate = JArray(np.zeros((5, *Q.shape[1:])))
        launch(k["prim2c"], (int(P.nx) + 2 * NG, int(P.ny) + 2 * NG, int(P.nz) + 2 * NG), Ustate, Qj)
    U = JArray(np.zeros((5, *Q.shape[1:]), dtype))
    _advance(k, P, Qj, m, S, Jj, U, np.float32(1) if typed else 1.0, xyz, Ustate)
    return U.a

"""Runtime for the reference's Julia kernels translated by jl2py.py (test infrastructure).

The translated kernels keep the reference's statements; this module gives them what CUDA.jl
and run.jl gave them:
- arrays taking Julia's 1-based, column-major subscripts A[i, j, k, n] over this
  repository's [n, k, j, i] layout (JArray);
- the thread index of a launch (one thread at a time: blockIdx = blockDim = 1,
  threadIdx = (i, j, k)) and Julia's max / min (a NaN wins), sqrt (NaN below 0), ifelse,
  zero, eps(Float32);
- the global constants of run.jl:8-13, 57-77 (γ, Rg, Cp, C_s, T_s, Pr, Ncons, the hybrid
  thresholds, Linear, NG, Nxp, Nyp, Nzp) from an f3d_params;
- the launch sequence of one finite-difference RHS: the sensor (solver.jl:424), the split and
  the reconstruction of each direction (solver.jl:133-188), the viscous fluxes and div
  (solver.jl:429) with U = 0 and dt = 1, so U ends holding J times the flux divergence, the RHS.

Every value is a Python float (binary64): the reference's algorithm in FP64, in its own
operation order. Slow (one Python call per thread): grids of a few hundred cells.
"""
from __future__ import annotations

import math
import unicodedata
from pathlib import Path
from types import SimpleNamespace

import numpy as np

NG = 4


class JArray:
    """A[i, j, k, n] (1-based, Julia's order) over a numpy array stored [n, k, j, i]."""

    __slots__ = ("a",)

    def __init__(self, a: np.ndarray):
        self.a = a

    def __getitem__(self, idx):
        if not isinstance(idx, tuple):
            return float(self.a[idx - 1])
        return float(self.a[tuple(x - 1 for x in reversed(idx))])

    def __setitem__(self, idx, v):
        if not isinstance(idx, tuple):
            self.a[idx - 1] = v
        else:
            self.a[tuple(x - 1 for x in reversed(idx))] = v

    def _fill(self, v):
        self.a[...] = v


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
    return math.sqrt(x) if x >= 0 else float("nan")


def _mat(r, c=None):
    return JArray(np.zeros(r if c is None else (c, r)))


HELPERS = dict(
    blockIdx=lambda: _one, blockDim=lambda: _one, threadIdx=lambda: _thread,
    max=_jmax, min=_jmin, sqrt=_sqrt, abs=abs,
    ifelse=lambda c, a, b: a if c else b, zero=lambda a: 0.0,
    _eps32=lambda: 2.0 ** -23, _mat=_mat, _f32=float, _f64=float,
    _p2=lambda x: x * x, _p3=lambda x: x * x * x,  # Julia's literal powers (Base.literal_pow)
)


def kernels(module_path: Path | str, P) -> dict:
    """The translated kernels with the run.jl constants of the parameter set P."""
    g = dict(HELPERS)
    gamma, rg = float(P.gamma), float(P.rg)
    up7 = [-3 / 420, 25 / 420, -101 / 420, 319 / 420, 214 / 420, -38 / 420, 4 / 420]
    cd6 = [0.0, 1 / 60, -2 / 15, 37 / 60, 37 / 60, -2 / 15, 1 / 60]
    lp = float(P.linear_phi)
    g.update({
        "γ": gamma, "Rg": rg, "Cp": float(P.cp) if P.cp else rg * gamma / (gamma - 1),
        "C_s": float(P.c_s), "T_s": float(P.t_s), "Pr": float(P.pr),
        "Ncons": 5, "Nprim": 6, "NG": NG, "Nxp": int(P.nx), "Nyp": int(P.ny), "Nzp": int(P.nz),
        "hybrid_ϕ1": float(P.phi1), "hybrid_ϕ2": float(P.phi2), "hybrid_ϕ3": float(P.phi3),
        "Linear": JArray(np.array([u * lp + c * (1.0 - lp) for u, c in zip(up7, cd6)])),
        "LES_smag": False, "LES_wale": False,
    })
    # Python reads identifiers NFKC-normalised (the ϕ of hybrid_ϕ1 becomes φ): so must the names
    g = {unicodedata.normalize("NFKC", name): v for name, v in g.items()}
    exec(compile(Path(module_path).read_text(), str(module_path), "exec"), g)
    return g


def launch(fn, ext, *args):
    """Every thread (i, j, k) of a grid covering ext = (X, Y, Z), one after the other."""
    X, Y, Z = ext
    for k in range(1, Z + 1):
        for j in range(1, Y + 1):
            for i in range(1, X + 1):
                _thread.x, _thread.y, _thread.z = i, j, k
                fn(*args)


SPLITS = ("fluxSplit_SW", "fluxSplit_LF", "fluxSplit_VL", "fluxSplit_AUSM")


def rhs(module_path, P, Q: np.ndarray, metrics: np.ndarray, J: np.ndarray) -> np.ndarray:
    """dU/dt at the interior (zero elsewhere) of the reference's finite-difference RHS from
    the ghost-filled primitive state Q (6, Nt...), the nine J^-1-scaled metrics and J."""
    k = kernels(module_path, P)
    nx, ny, nz = int(P.nx), int(P.ny), int(P.nz)
    ext = (nx + 2 * NG, ny + 2 * NG, nz + 2 * NG)
    Qj, Jj = JArray(Q.astype(np.float64)), JArray(J.astype(np.float64))
    m = [JArray(metrics[n].astype(np.float64)) for n in range(9)]
    # solver.jl:286-288: s = sqrt(a^2 + b^2 + c^2) of each metric row
    S = [JArray(np.sqrt(metrics[3 * d] ** 2 + metrics[3 * d + 1] ** 2 + metrics[3 * d + 2] ** 2)) for d in range(3)]
    phi = JArray(np.zeros(Q.shape[1:]))
    launch(k["shockSensor"], ext, phi, Qj)
    Fp, Fm = JArray(np.zeros((5, *Q.shape[1:]))), JArray(np.zeros((5, *Q.shape[1:])))
    F = [JArray(np.zeros((5, nz, ny, nx + 1))), JArray(np.zeros((5, nz, ny + 1, nx))),
         JArray(np.zeros((5, nz + 1, ny, nx)))]
    split = k[SPLITS[int(P.split_method)]]
    for d, name in enumerate("xyz"):
        launch(split, ext, Qj, Fp, Fm, S[d], m[3 * d], m[3 * d + 1], m[3 * d + 2])
        if int(P.character):
            launch(k["advect_" + name + "c"], ext, F[d], phi, S[d], Fp, Fm, Qj, m[3 * d], m[3 * d + 1], m[3 * d + 2])
        else:
            launch(k["advect_" + name], ext, F[d], phi, S[d], Fp, Fm, 5)
    Fv = [JArray(np.zeros((4, nz + 4, ny + 4, nx + 4))) for _ in range(3)]
    if int(P.viscous):
        launch(k["viscousFlux"], ext, *Fv, Qj, *m, Jj)
    U = JArray(np.zeros((5, *Q.shape[1:])))
    launch(k["div"], (nx, ny, nz), U, *F, *Fv, 1.0, Jj)
    return U.a

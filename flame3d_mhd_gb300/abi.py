"""ctypes binding of libflame3d_gpu.so (the C ABI declared in include/flame3d_gpu.h).

The structures mirror f3d_bc and f3d_params field for field. load() finds the in-tree
library built by flame3d_mhd_gb300.build and raises if it is missing: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

F3D_OK = 0
F3D_ERR_ARG = 1
F3D_ERR_ALIGN = 2
F3D_ERR_CUDA = 3
F3D_ERR_NONFINITE = 4
F3D_ERR_UNSUPPORTED = 5
F3D_ERR_STATE = 6
F3D_ERR_TOO_LARGE = 7
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024

SPLIT_SW, SPLIT_LF, SPLIT_VL, SPLIT_AUSM = 0, 1, 2, 3
SPLIT_NAMES = {"SW": SPLIT_SW, "LF": SPLIT_LF, "VL": SPLIT_VL, "AUSM": SPLIT_AUSM}
PREC_FP64, PREC_MIXED, PREC_REF32 = 0, 1, 2
METRICS_READFORT, METRICS_PARSE_MESH = 0, 1  # coefficient sets of f3d_compute_metrics_f32
SCHEME_FDM, SCHEME_FVM_EIGEN, SCHEME_FVM_CONS = 0, 1, 2
FILTER_NONE, FILTER_LINEAR, FILTER_NONLINEAR = 0, 1, 2
LES_NONE, LES_SMAGORINSKY, LES_WALE = 0, 1, 2
BC_PERIODIC, BC_DIRICHLET, BC_ZERO_GRADIENT, BC_WALL_ADIABATIC, BC_WALL_ISOTHERMAL = 0, 1, 2, 3, 4
BC_INFLOW_PROFILE = 5

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libflame3d_gpu.so"


class F3DBc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad_", C.c_int32), ("rho", C.c_double), ("u", C.c_double),
                ("v", C.c_double), ("w", C.c_double), ("p", C.c_double), ("t_wall", C.c_double)]


class F3DParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("ng", C.c_int32),
                ("gamma", C.c_double), ("rg", C.c_double), ("cp", C.c_double), ("c_s", C.c_double),
                ("t_s", C.c_double), ("pr", C.c_double), ("phi1", C.c_double), ("phi2", C.c_double),
                ("phi3", C.c_double), ("linear_phi", C.c_double), ("clamp_eps", C.c_double),
                ("split_method", C.c_int32), ("character", C.c_int32), ("viscous", C.c_int32),
                ("precision", C.c_int32), ("bc", F3DBc * 6), ("scheme", C.c_int32), ("adjoint_lean", C.c_int32),
                ("lts", C.c_int32), ("filter", C.c_int32), ("filter_interval", C.c_int32), ("les", C.c_int32),
                ("lts_cfl", C.c_double), ("filter_s0", C.c_double), ("filter_rth", C.c_double)]


def params_to_dict(p: F3DParams) -> dict:
    d = {f: getattr(p, f) for f, _ in F3DParams._fields_ if f != "bc"}
    d["bc"] = [{f: getattr(b, f) for f, _ in F3DBc._fields_ if f != "pad_"} for b in p.bc]
    return d


def make_params(nx: int, ny: int, nz: int, **kw) -> F3DParams:
    """Reference defaults (run.jl:3-77, boundary.jl BCs) for an nx*ny*nz grid, then overrides.

    Scalar overrides use the f3d_params field names; `split` accepts "SW"/"LF"/"VL"/"AUSM";
    `bc` takes a list of six dicts (x-, x+, y-, y+, z-, z+) with keys kind, rho, u, v, w, p,
    t_wall. The defaults are set in Python (not through the library) so that the oracle
    can build parameters on a machine without the CUDA library.
    """
    p = F3DParams()
    p.nx, p.ny, p.nz, p.ng = nx, ny, nz, 4
    p.gamma, p.rg, p.cp, p.c_s, p.t_s, p.pr = 1.4, 287.0, 0.0, 1.458e-6, 110.4, 0.72
    p.phi1, p.phi2, p.phi3, p.linear_phi, p.clamp_eps = 0.05, 1.0, 10.0, 1.0, 0.0
    p.split_method, p.character, p.viscous, p.precision = SPLIT_SW, 1, 1, PREC_FP64
    p.lts_cfl, p.filter_interval, p.filter_rth, p.filter_s0 = 0.5, 100, 1e-5, 1.0  # run.jl:22, 52-54
    fs = dict(kind=BC_DIRICHLET, rho=1.0, u=0.5, v=0.0, w=0.0, p=1.0 / 1.4)
    bcs = [fs, dict(kind=BC_ZERO_GRADIENT), dict(kind=BC_WALL_ADIABATIC), fs,
           dict(kind=BC_PERIODIC), dict(kind=BC_PERIODIC)]
    if "split" in kw:
        s = kw.pop("split")
        p.split_method = SPLIT_NAMES[s] if isinstance(s, str) else int(s)
    if "bc" in kw:
        bcs = kw.pop("bc")
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(f"unknown f3d_params field {k!r}")
        setattr(p, k, v)
    for f, b in enumerate(bcs):
        p.bc[f] = F3DBc()
        for k, v in b.items():
            setattr(p.bc[f], k, v)
    return p


_lib = None


def load() -> C.CDLL:
    """Load the in-tree CUDA library once. Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with flame3d_mhd_gb300.build.build()")
    lib = C.CDLL(str(LIB_PATH))
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    P = C.POINTER(F3DParams)
    sigs = {
        "f3d_version": (ip, []),
        "f3d_default_params": (ip, [ip, ip, ip, P]),
        "f3d_create": (ip, [P, C.POINTER(vp)]),
        "f3d_destroy": (ip, [vp]),
        "f3d_last_error": (C.c_char_p, [vp]),
        "f3d_scratch_bytes": (ip, [vp, C.POINTER(C.c_size_t)]),
        "f3d_set_metrics": (ip, [vp, vp * 9, vp, vp]),
        "f3d_compute_metrics": (ip, [vp, vp, vp, vp, vp * 9, vp, vp]),
        "f3d_c2prim": (ip, [vp, vp, vp, vp]),
        "f3d_prim2c": (ip, [vp, vp, vp, vp]),
        "f3d_lincomb": (ip, [vp, vp, vp, C.c_double, C.c_double, vp]),
        "f3d_fill_ghosts": (ip, [vp, vp, vp, vp]),
        "f3d_rhs": (ip, [vp, vp, vp, vp]),
        "f3d_rk3_stage": (ip, [vp, ip, C.c_double, vp, vp, vp, vp]),
        "f3d_rk3_steps": (ip, [vp, ip, C.c_double, vp, vp, vp, vp]),
        "f3d_rk3_step": (ip, [vp, C.c_double, vp, vp, vp, vp]),
        "f3d_cfl_dt": (ip, [vp, vp, C.c_double, dp, vp]),
        "f3d_check_finite": (ip, [vp, vp, vp]),
        "f3d_debug_sensor": (ip, [vp, vp, vp, vp]),
        "f3d_debug_split": (ip, [vp, ip, vp, vp, vp, vp]),
        "f3d_debug_face_flux": (ip, [vp, ip, vp, vp, vp, vp]),
        "f3d_debug_viscous": (ip, [vp, vp, vp, vp, vp, vp]),
        "f3d_div": (ip, [vp, vp, vp, vp, vp, vp, vp, vp, C.c_double, vp]),
        "f3d_measure_pipes": (ip, [dp, dp]),
        "f3d_kernel_count": (ip, []),
        "f3d_kernel_name": (C.c_char_p, [ip]),
        "f3d_profile_step": (ip, [vp, C.c_double, vp, vp, vp, vp, dp, C.POINTER(C.c_int)]),
        "f3d_rhs_noalloc": (ip, [P, vp * 9, vp, vp, vp, vp]),
        "f3d_rhs_vjp": (ip, [vp, vp, vp, vp, vp]),
        "f3d_rk3_step_vjp": (ip, [vp, C.c_double, vp, vp, vp, vp]),
        "f3d_set_inflow_profile": (ip, [vp, ip, vp, vp]),
        "f3d_set_coordinates": (ip, [vp, vp, vp, vp, vp]),
        "f3d_filter": (ip, [vp, vp, vp, vp, vp]),
        "f3d_local_dt": (ip, [vp, vp, vp, vp]),
        "f3d_debug_round_f32": (ip, [vp, vp, C.c_longlong, vp]),
        "f3d_set_inflow_profile_cotangent": (ip, [vp, ip, vp, vp]),
        "f3d_rk3_step_vjp_stages": (ip, [vp, C.c_double, vp, vp, vp, vp, vp, vp]),
        "f3d_set_metrics_f32": (ip, [vp, vp * 9, vp, vp]),
        "f3d_compute_metrics_f32": (ip, [vp, vp, vp, vp, vp * 9, vp, ip, vp]),
        "f3d_set_metrics_cotangent": (ip, [vp, C.c_void_p, vp, vp]),
        "f3d_c2prim_f32": (ip, [vp, vp, vp, vp]),
        "f3d_prim2c_f32": (ip, [vp, vp, vp, vp]),
        "f3d_fill_ghosts_f32": (ip, [vp, vp, vp, vp]),
        "f3d_rhs_f32": (ip, [vp, vp, vp, vp]),
        "f3d_rk3_stage_f32": (ip, [vp, ip, C.c_float, vp, vp, vp, vp]),
        "f3d_rk3_steps_f32": (ip, [vp, ip, C.c_float, vp, vp, vp, vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# every symbol the header declares (checked by the CPU test suite)
EXPORTED = ["f3d_version", "f3d_default_params", "f3d_create", "f3d_destroy", "f3d_last_error",
            "f3d_scratch_bytes", "f3d_set_metrics", "f3d_compute_metrics", "f3d_c2prim", "f3d_prim2c",
            "f3d_lincomb", "f3d_fill_ghosts", "f3d_rhs", "f3d_rk3_stage", "f3d_rk3_steps", "f3d_cfl_dt",
            "f3d_check_finite", "f3d_debug_sensor", "f3d_debug_split", "f3d_debug_face_flux",
            "f3d_debug_viscous", "f3d_div", "f3d_measure_pipes", "f3d_kernel_count", "f3d_kernel_name",
            "f3d_profile_step", "f3d_rhs_noalloc", "f3d_rhs_vjp", "f3d_rk3_step_vjp", "f3d_set_inflow_profile",
            "f3d_set_coordinates", "f3d_filter", "f3d_local_dt", "f3d_debug_round_f32",
            "f3d_set_inflow_profile_cotangent", "f3d_rk3_step_vjp_stages", "f3d_set_metrics_f32",
            "f3d_c2prim_f32", "f3d_prim2c_f32", "f3d_fill_ghosts_f32", "f3d_rhs_f32", "f3d_rk3_stage_f32",
            "f3d_rk3_steps_f32", "f3d_set_metrics_cotangent", "f3d_compute_metrics_f32", "f3d_rk3_step"]


class F3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"flame3d status {code}: {msg}")
        self.code = code

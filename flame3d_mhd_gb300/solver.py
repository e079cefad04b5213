"""Host-side mirror of the reference's finite-difference solver interface over the C ABI.

Method names and argument meaning follow the reference's Julia functions (solver.jl,
utils.jl, boundary.jl, schemes.jl, div.jl): prim2c(U, Q), c2Prim(U, Q), linComb(U, Un, a, b),
fillGhost(Q, U) (exchange_ghost + fillGhost), shockSensor(phi, Q), flowAdvance(Q),
div(U, Fx, Fy, Fz, Fv_x, Fv_y, Fv_z, dt) and the RK3 loop of time_step. Arrays are torch
float64 CUDA tensors (float32 for an F3D_PREC_REF32 context, the reference's own Float32
arrays) whose memory is the reference's Julia layout: a tensor of shape
(nvar, Nz+8, Ny+8, Nx+8) in C order is the Julia array (Nx+8, Ny+8, Nz+8, nvar).

PyTorch only provides device memory and the stream here; every computation runs in the
CUDA kernels of libflame3d_gpu.so, and a missing library or a non-CUDA tensor raises.
"""
from __future__ import annotations

import contextlib
import ctypes as C

import torch

from . import abi
from .abi import F3DError, F3DParams

NG = 4


@contextlib.contextmanager
def side_stream(stream: torch.cuda.Stream | None = None):
    """Run the enclosed calls on a side stream (f3d_rk3_steps captures its step into a CUDA
    graph only on a non-default stream), ordered after the work already queued on the
    current stream; on exit the current stream is ordered after the side stream's work.
    PyTorch's pool streams are non-blocking: without these waits the side stream's kernels
    could start before the set-up launched on the default stream (metrics, ghost fill,
    host-to-device copies) has finished."""
    cur = torch.cuda.current_stream()
    s = stream if stream is not None else torch.cuda.Stream()
    s.wait_stream(cur)
    with torch.cuda.stream(s):
        yield s
    cur.wait_stream(s)


class Flame3D:
    """One solver context (f3d_create) for a fixed grid and parameter set."""

    def __init__(self, params: F3DParams, device: int | torch.device | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("Flame3D needs a CUDA device; there is no CPU path")
        self.lib = abi.load()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else
                                   torch.device(device).index or 0)
        self.params = params
        # F3D_PREC_REF32: the reference's Float32 arrays (the *_f32 entries)
        self.ref32 = params.precision == abi.PREC_REF32
        self.dtype = torch.float32 if self.ref32 else torch.float64
        self.nx, self.ny, self.nz = params.nx, params.ny, params.nz
        self.shape3 = (self.nz + 2 * NG, self.ny + 2 * NG, self.nx + 2 * NG)
        self.metrics = None
        self.J = None
        with torch.cuda.device(self.device):
            h = C.c_void_p()
            rc = self.lib.f3d_create(C.byref(params), C.byref(h))
            if rc != abi.F3D_OK:
                raise F3DError(rc, "f3d_create rejected the parameters (see stderr)")
            self._h = h

    # ---- plumbing -------------------------------------------------------------------
    def _check(self, rc: int):
        if rc != abi.F3D_OK:
            raise F3DError(rc, self.lib.f3d_last_error(self._h).decode())

    def _stream(self) -> C.c_void_p:
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _ptr(self, t: torch.Tensor | None, nvar: int | None = None) -> C.c_void_p | None:
        if t is None:
            return None
        if not (t.is_cuda and t.dtype == self.dtype and t.is_contiguous()):
            raise TypeError(f"arrays must be contiguous {str(self.dtype)[6:]} CUDA tensors")
        if nvar is not None and tuple(t.shape) != (nvar, *self.shape3) and not (
                nvar == 1 and tuple(t.shape) == self.shape3):
            raise ValueError(f"expected shape {(nvar, *self.shape3)}, got {tuple(t.shape)}")
        return C.c_void_p(t.data_ptr())

    def field(self, nvar: int) -> torch.Tensor:
        """Zero-initialised array in the reference layout with nvar variables."""
        shape = self.shape3 if nvar == 1 else (nvar, *self.shape3)
        return torch.zeros(shape, dtype=self.dtype, device=self.device)

    def face_field(self, d: int) -> torch.Tensor:
        """Zero array shaped like the reference's Fx / Fy / Fz (solver.jl:298-300)."""
        n = [self.nz, self.ny, self.nx]
        n[2 - d] += 1
        return torch.zeros((5, *n), dtype=torch.float64, device=self.device)

    def viscous_field(self) -> torch.Tensor:
        """Zero array shaped like Fv_x / Fv_y / Fv_z (solver.jl:301-303)."""
        return torch.zeros((4, self.nz + NG, self.ny + NG, self.nx + NG), dtype=torch.float64, device=self.device)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.f3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scratch_bytes(self) -> int:
        b = C.c_size_t()
        self._check(self.lib.f3d_scratch_bytes(self._h, C.byref(b)))
        return b.value

    # ---- geometry ---------------------------------------------------------------------
    def set_metrics(self, metrics: list[torch.Tensor], J: torch.Tensor):
        """Nine J^-1-scaled metrics in metrics.h5 order and J (solver.jl:238-288)."""
        if len(metrics) != 9:
            raise ValueError("need nine metric arrays")
        arr = (C.c_void_p * 9)(*[self._ptr(m, 1) for m in metrics])
        fn = self.lib.f3d_set_metrics_f32 if self.ref32 else self.lib.f3d_set_metrics
        self._check(fn(self._h, arr, self._ptr(J, 1), self._stream()))
        self.metrics, self.J = list(metrics), J  # keep the borrowed arrays alive

    def filter(self, U: torch.Tensor, Un: torch.Tensor, Q: torch.Tensor):
        """One pass of the explicit filter of params.filter (linearFilter_x/y/z, or pre_x/y/z
        and filter_x/y/z) over U; Un receives the per-direction copies (solver.jl:446-470)."""
        self._check(self.lib.f3d_filter(self._h, self._ptr(U, 5), self._ptr(Un, 5), self._ptr(Q, 6), self._stream()))

    def compute_dt(self, Q: torch.Tensor, dt: torch.Tensor | None = None) -> torch.Tensor:
        """Local time step of every interior cell (utils.jl:73-99)."""
        if dt is None:
            dt = self.field(1)
        self._check(self.lib.f3d_local_dt(self._h, self._ptr(Q, 6), self._ptr(dt, 1), self._stream()))
        return dt

    def set_coordinates(self, x: torch.Tensor, y: torch.Tensor, z: torch.Tensor):
        """Ghost-filled cell-centre coordinates for the finite-volume schemes: face normals
        and areas (FVM.jl:16-29) are computed from them once (a no-op for the FDM scheme)."""
        self._check(self.lib.f3d_set_coordinates(self._h, self._ptr(x, 1), self._ptr(y, 1), self._ptr(z, 1),
                                                 self._stream()))

    def set_inflow_profile_cotangent(self, face: int, prof_bar: torch.Tensor | None):
        """Accumulate dJ/d(profile of face) into prof_bar during the adjoint calls (None stops)."""
        if prof_bar is None:
            self._check(self.lib.f3d_set_inflow_profile_cotangent(self._h, face, None, self._stream()))
            return
        if (tuple(prof_bar.shape) != self.profile_shape(face) or prof_bar.dtype != torch.float64
                or not prof_bar.is_cuda or not prof_bar.is_contiguous()):
            raise ValueError(f"expected a contiguous float64 CUDA tensor of shape {self.profile_shape(face)}")
        self._check(self.lib.f3d_set_inflow_profile_cotangent(self._h, face, C.c_void_p(prof_bar.data_ptr()),
                                                              self._stream()))
        self._profile_bars = getattr(self, "_profile_bars", {})
        self._profile_bars[face] = prof_bar

    def set_metrics_cotangent(self, metrics_bar: list[torch.Tensor] | None, J_bar: torch.Tensor | None = None):
        """Accumulate dJ/d(metrics) and dJ/dJ into the nine arrays and J_bar during the
        adjoint calls (None stops)."""
        if metrics_bar is None:
            self._check(self.lib.f3d_set_metrics_cotangent(self._h, None, None, self._stream()))
            self._metric_bars = None
            return
        if len(metrics_bar) != 9:
            raise ValueError("need nine metric cotangent arrays")
        arr = (C.c_void_p * 9)(*[self._ptr(m, 1) for m in metrics_bar])
        self._check(self.lib.f3d_set_metrics_cotangent(self._h, C.cast(arr, C.c_void_p), self._ptr(J_bar, 1),
                                                       self._stream()))
        self._metric_bars = (list(metrics_bar), J_bar, arr)

    def profile_shape(self, face: int) -> tuple[int, int, int]:
        """(5, Tb, Ta) of an inflow-profile face: its transverse extent including ghosts."""
        nxt, nyt, nzt = self.shape3[2], self.shape3[1], self.shape3[0]
        d = face // 2
        return (5, nzt, nyt) if d == 0 else ((5, nzt, nxt) if d == 1 else (5, nyt, nxt))

    def set_inflow_profile(self, face: int, prof: torch.Tensor):
        """Per-point (rho, u, v, w, p) of an F3D_BC_INFLOW_PROFILE face (borrowed)."""
        if not (prof.is_cuda and prof.dtype == torch.float64 and prof.is_contiguous()):
            raise TypeError("profile must be a contiguous float64 CUDA tensor")
        if tuple(prof.shape) != self.profile_shape(face):
            raise ValueError(f"expected shape {self.profile_shape(face)}, got {tuple(prof.shape)}")
        self._check(self.lib.f3d_set_inflow_profile(self._h, face, C.c_void_p(prof.data_ptr()), self._stream()))
        self._profiles = getattr(self, "_profiles", {})
        self._profiles[face] = prof  # keep the borrowed array alive

    def compute_metrics(self, x: torch.Tensor, y: torch.Tensor, z: torch.Tensor,
                        coefficients: int = abi.METRICS_READFORT):
        """Metrics and J from coordinates on the device: in FP64 (parse_mesh.jl:139-248), or
        in the Float32 form the reference's own Float32 set-up metrics with the coefficients
        of readfort.jl or parse_mesh.jl (bitwise those of its metrics.h5)."""
        ms = [self.field(1) for _ in range(9)]
        J = self.field(1)
        arr = (C.c_void_p * 9)(*[self._ptr(m, 1) for m in ms])
        xyz = (self._ptr(x, 1), self._ptr(y, 1), self._ptr(z, 1))
        if self.ref32:
            self._check(self.lib.f3d_compute_metrics_f32(self._h, *xyz, arr, self._ptr(J, 1), coefficients,
                                                         self._stream()))
        else:
            self._check(self.lib.f3d_compute_metrics(self._h, *xyz, arr, self._ptr(J, 1), self._stream()))
        return ms, J

    # ---- utils.jl / boundary.jl ----------------------------------------------------------
    def prim2c(self, U: torch.Tensor, Q: torch.Tensor):
        fn = self.lib.f3d_prim2c_f32 if self.ref32 else self.lib.f3d_prim2c
        self._check(fn(self._h, self._ptr(Q, 6), self._ptr(U, 5), self._stream()))

    def c2Prim(self, U: torch.Tensor, Q: torch.Tensor):
        fn = self.lib.f3d_c2prim_f32 if self.ref32 else self.lib.f3d_c2prim
        self._check(fn(self._h, self._ptr(U, 5), self._ptr(Q, 6), self._stream()))

    def linComb(self, U: torch.Tensor, Un: torch.Tensor, a: float, b: float):
        self._check(self.lib.f3d_lincomb(self._h, self._ptr(U, 5), self._ptr(Un, 5), a, b, self._stream()))

    def fillGhost(self, Q: torch.Tensor, U: torch.Tensor):
        """exchange_ghost (periodic, one GPU) followed by fillGhost for Q and U."""
        fn = self.lib.f3d_fill_ghosts_f32 if self.ref32 else self.lib.f3d_fill_ghosts
        self._check(fn(self._h, self._ptr(Q, 6), self._ptr(U, 5), self._stream()))

    # ---- schemes.jl / split.jl / viscous.jl / div.jl --------------------------------------
    def shockSensor(self, phi: torch.Tensor, Q: torch.Tensor):
        self._check(self.lib.f3d_debug_sensor(self._h, self._ptr(Q, 6), self._ptr(phi, 1), self._stream()))

    def fluxSplit(self, d: int, Q: torch.Tensor, Fp: torch.Tensor, Fm: torch.Tensor):
        self._check(self.lib.f3d_debug_split(self._h, d, self._ptr(Q, 6), self._ptr(Fp, 5), self._ptr(Fm, 5),
                                             self._stream()))

    def advect(self, d: int, F: torch.Tensor, phi: torch.Tensor | None, Q: torch.Tensor):
        """Face flux of direction d in the shape of Fx/Fy/Fz (advect_x/xc ... advect_z/zc)."""
        self._check(self.lib.f3d_debug_face_flux(self._h, d, self._ptr(Q, 6), self._ptr(phi, 1), self._ptr(F),
                                                 self._stream()))

    def viscousFlux(self, Fv_x: torch.Tensor, Fv_y: torch.Tensor, Fv_z: torch.Tensor, Q: torch.Tensor):
        self._check(self.lib.f3d_debug_viscous(self._h, self._ptr(Q, 6), self._ptr(Fv_x), self._ptr(Fv_y),
                                               self._ptr(Fv_z), self._stream()))

    def flowAdvance(self, Q: torch.Tensor, phi: torch.Tensor | None = None):
        """Face and viscous fluxes of one stage (solver.jl:133-188): (Fx, Fy, Fz, Fv_x, Fv_y, Fv_z)."""
        if phi is None:
            phi = self.field(1)
            self.shockSensor(phi, Q)
        F = [self.face_field(d) for d in range(3)]
        for d in range(3):
            self.advect(d, F[d], phi, Q)
        Fv = [self.viscous_field() for _ in range(3)] if self.params.viscous else [None] * 3
        if self.params.viscous:
            self.viscousFlux(*Fv, Q)
        return (*F, *Fv)

    def div(self, U, Fx, Fy, Fz, Fv_x, Fv_y, Fv_z, dt: float):
        self._check(self.lib.f3d_div(self._h, self._ptr(U, 5), self._ptr(Fx), self._ptr(Fy), self._ptr(Fz),
                                     self._ptr(Fv_x), self._ptr(Fv_y), self._ptr(Fv_z), dt, self._stream()))

    # ---- fused paths ----------------------------------------------------------------
    def rhs(self, Q: torch.Tensor, dUdt: torch.Tensor | None = None) -> torch.Tensor:
        """L(U) at interior cells from a ghost-filled Q (fused sensor/split/reconstruction/divergence)."""
        if dUdt is None:
            dUdt = self.field(5)
        fn = self.lib.f3d_rhs_f32 if self.ref32 else self.lib.f3d_rhs
        self._check(fn(self._h, self._ptr(Q, 6), self._ptr(dUdt, 5), self._stream()))
        return dUdt

    def rk3_stage(self, stage: int, dt: float, U, Un, Q):
        fn = self.lib.f3d_rk3_stage_f32 if self.ref32 else self.lib.f3d_rk3_stage
        self._check(fn(self._h, stage, dt, self._ptr(U, 5), self._ptr(Un, 5), self._ptr(Q, 6), self._stream()))

    def time_step(self, U, Un, Q, dt: float, nsteps: int):
        """nsteps SSP-RK3 steps (the hot loop of solver.jl:410-444)."""
        fn = self.lib.f3d_rk3_steps_f32 if self.ref32 else self.lib.f3d_rk3_steps
        self._check(fn(self._h, nsteps, dt, self._ptr(U, 5), self._ptr(Un, 5), self._ptr(Q, 6), self._stream()))

    # ---- discrete adjoint ----------------------------------------------------------
    def rhs_vjp(self, U: torch.Tensor, Lbar: torch.Tensor, Ubar: torch.Tensor | None = None) -> torch.Tensor:
        """(dL/dU)^T Lbar for L(U) = RHS(ghost-filled c2Prim(U)), interior cells."""
        if Ubar is None:
            Ubar = self.field(5)
        self._check(self.lib.f3d_rhs_vjp(self._h, self._ptr(U, 5), self._ptr(Lbar, 5), self._ptr(Ubar, 5),
                                         self._stream()))
        return Ubar

    def rk3_step_vjp(self, dt: float, U0: torch.Tensor, Ubar_next: torch.Tensor,
                     Ubar: torch.Tensor | None = None, Ustage: torch.Tensor | None = None,
                     Lbar_stage: torch.Tensor | None = None) -> torch.Tensor:
        """Cotangent of the state at the start of one SSP-RK3 step from the one at its end.
        Ustage / Lbar_stage, shape (3, 5, Nzt, Nyt, Nxt) when given, receive the three stage
        states and the cotangents of their RHS values (interior cells)."""
        if Ubar is None:
            Ubar = self.field(5)
        if Ustage is None and Lbar_stage is None:
            self._check(self.lib.f3d_rk3_step_vjp(self._h, dt, self._ptr(U0, 5), self._ptr(Ubar_next, 5),
                                                  self._ptr(Ubar, 5), self._stream()))
            return Ubar
        opt = [None if t is None else C.c_void_p(self._stages_ptr(t)) for t in (Ustage, Lbar_stage)]
        self._check(self.lib.f3d_rk3_step_vjp_stages(self._h, dt, self._ptr(U0, 5), self._ptr(Ubar_next, 5),
                                                     self._ptr(Ubar, 5), opt[0], opt[1], self._stream()))
        return Ubar

    def _stages_ptr(self, t: torch.Tensor) -> int:
        want = (3, 5, *self.shape3)
        if tuple(t.shape) != want or t.dtype != torch.float64 or not t.is_contiguous() or not t.is_cuda:
            raise ValueError(f"expected a contiguous float64 CUDA tensor of shape {want}")
        return t.data_ptr()

    def q_from_u(self, U: torch.Tensor, Q: torch.Tensor | None = None) -> torch.Tensor:
        """Q = c2Prim(U) with its ghost layers (and U's) filled: the stage input of solver.jl."""
        if Q is None:
            Q = self.field(6)
        self.c2Prim(U, Q)
        self.fillGhost(Q, U)
        return Q

    def profile_step(self, U, Un, Q, dt: float) -> dict:
        """One RK3 step with per-launch CUDA events: {kernel name: (ms, launches)}."""
        n = self.lib.f3d_kernel_count()
        ms = (C.c_double * n)()
        cnt = (C.c_int * n)()
        self._check(self.lib.f3d_profile_step(self._h, dt, self._ptr(U, 5), self._ptr(Un, 5), self._ptr(Q, 6),
                                              self._stream(), ms, cnt))
        return {self.lib.f3d_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n) if cnt[k]}

    def cfl_dt(self, Q: torch.Tensor, cfl: float) -> float:
        out = C.c_double()
        self._check(self.lib.f3d_cfl_dt(self._h, self._ptr(Q, 6), cfl, C.byref(out), self._stream()))
        return out.value

    def check_finite(self, U: torch.Tensor) -> bool:
        rc = self.lib.f3d_check_finite(self._h, self._ptr(U, 5), self._stream())
        if rc == abi.F3D_ERR_NONFINITE:
            return False
        self._check(rc)
        return True


def measure_pipes() -> tuple[float, float]:
    """(FP64, FP32) FMA throughput of the current device in TFLOP/s."""
    lib = abi.load()
    a, b = C.c_double(), C.c_double()
    rc = lib.f3d_measure_pipes(C.byref(a), C.byref(b))
    if rc != abi.F3D_OK:
        raise F3DError(rc, "f3d_measure_pipes failed")
    return a.value, b.value

"""Make tests/golden/jl_reference_rhs.npz: the reference's own finite-difference RHS, from its
Julia kernels translated mechanically into Python (oracle/ref_jl/jl2py.py) and run on the CPU
(oracle/ref_jl/runtime.py), on
- the inputs of the golden fixtures (test_oracle.py::test_golden_fixtures: four splits,
  characteristic and component-wise, hybrid and WENO5-everywhere, periodic, reference and
  mixed boundary rules; inviscid), and
- five viscous cases made here the same way (curvilinear random states, Sutherland viscosity
  large enough for the viscous terms to matter; two with the LES closures, Smagorinsky and
  WALE), whose inputs are stored too;
and, for the cases with boundary.jl's own boundary set, the reference's prim2c, c2Prim with
the ghost fill, and two SSP-RK3 steps (the stage loop of solver.jl); for the viscous cases its
local time step and one pass of each filter, and for those with boundary.jl's boundary set
two steps of the whole time_step loop (solver.jl:410-470) with local time stepping and/or
either filter (STEP_VARIANTS), as SHA-256 digests of U and Q; for every case a SHA-256 of the metrics and J of
parse_mesh.jl:139-248 from the coordinates (the arrays themselves are those stored with the
inputs);
- four finite-volume cases (FVM.jl, the reference's default scheme: Roe-characteristic and
  component-wise reconstruction, inviscid and viscous; noise that grows along x and two
  pressure spikes, so that faces of all four branches occur): the face fluxes of the three
  directions, the RHS and, for boundary.jl's boundary set, two SSP-RK3 steps, from the
  translation with jl2py.CORRECTIONS applied, and the face fluxes of the translation as
  written (two defects of FVM.jl: the corrected and as-written translations differ on the
  Roe-characteristic WENO5 faces and on the component-wise y and z faces only);
- the reference's Float32 arithmetic: the translation with Julia's types kept (jl2py typed:
  Float32 arrays, f0 literals and ::Float32 locals, the Float64 WENO7 epsilon and what it
  promotes) on the finite-difference cases' inputs rounded to Float32, as SHA-256 digests of
  the RHS and, for boundary.jl's boundary set, of prim2c, c2Prim with the ghost fill and two
  SSP-RK3 steps (Float32 dt and weights), and of the metrics of parse_mesh.jl:139-248 (Float32
  arrays, Float64 coefficients) and of SCU-benchmark/readfort.jl:104-208 (Float32 coefficients)
  on the coordinates rounded to Float32, all little-endian binary32;
- the ghost coordinates of readfort.jl's generateXYZ (:34-99, with ./= 1000) and of solver.jl's
  extrapolation, in binary64 and in Float32, on one grid whose interior is stored
  (ghosts__x/y/z), as SHA-256 digests; and parse_mesh.jl's flat-plate coordinates (:38-136) in
  Float32 on a 9 x 7 x 5 grid (its sinh taken in binary64 and rounded to Float32).
The file also records SHA-256 digests of the translated Julia files and of the generated
modules. Needs the reference tree (read only):

  python tests/golden/make_jl_reference.py --ref <reference tree>
"""
from __future__ import annotations

import argparse
import hashlib
import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from flame3d_mhd_gb300.abi import BC_PERIODIC, make_params  # noqa: E402
from flame3d_mhd_gb300.cases import params_copy  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle.ref_jl import jl2py, runtime  # noqa: E402

NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
VISCOUS = {
    "curvi_viscous_char_sw_periodic": dict(n=(7, 6, 6), params=dict(
        character=1, viscous=1, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0,
        bc=[dict(kind=BC_PERIODIC)] * 6), seed=35, spikes=4),
    "curvi_viscous_comp_lf_refbc": dict(n=(6, 6, 5), params=dict(
        character=0, viscous=1, split_method=1, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0),
        seed=36, spikes=4),
    "curvi_viscous_char_sw_refbc": dict(n=(6, 5, 5), params=dict(
        character=1, viscous=1, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0), seed=37, spikes=4),
    # the LES closures of viscous.jl:66-106 (run.jl:4-5 LES_smag / LES_wale)
    "curvi_les_smagorinsky_char_sw_refbc": dict(n=(6, 5, 5), params=dict(
        character=1, viscous=1, les=1, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0), seed=61, spikes=4),
    "curvi_les_wale_comp_ausm_periodic": dict(n=(6, 6, 5), params=dict(
        character=0, split_method=3, viscous=1, les=2, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0,
        bc=[dict(kind=BC_PERIODIC)] * 6), seed=62, spikes=4),
}
RK3_DT, RK3_STEPS = 2e-4, 2
# the time_step loop's options: compute_dt at the first stage and div_LTS, the filters after
# every filtering_interval-th step (LTS_CFL 1e-3 keeps the local steps of these rough random
# states near the fixed dt; at 0.3 they are about 1000 times larger and the states blow up)
STEP_VARIANTS = {
    "lts": dict(lts=1, lts_cfl=1e-3),
    "filter_linear": dict(filter=1, filter_interval=2, filter_s0=0.5),
    "filter_shock": dict(filter=2, filter_interval=1, filter_rth=1e-5, filter_s0=1.0),
    "lts_filter_shock": dict(lts=1, lts_cfl=1e-3, filter=2, filter_interval=2, filter_rth=1e-5, filter_s0=1.0),
}
FVM = {
    "fvm_eigen_refbc": dict(n=(6, 5, 5), params=dict(scheme=1, viscous=0), seed=51),
    "fvm_eigen_viscous_refbc": dict(n=(6, 5, 5), params=dict(scheme=1, viscous=1, c_s=1e-2, t_s=1.0), seed=52),
    "fvm_cons_refbc": dict(n=(6, 5, 5), params=dict(scheme=2, viscous=0), seed=53),
    "fvm_cons_viscous_periodic": dict(n=(6, 5, 5), params=dict(
        scheme=2, viscous=1, c_s=1e-2, t_s=1.0, bc=[dict(kind=BC_PERIODIC)] * 6), seed=54),
}
FVM_COMMON = dict(phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0)


def fvm_state(P, n, seed):
    """Primitive state with uniform noise whose amplitude grows from 1e-3 to 0.1 along x about
    (1, 0.2, 0.2, 0.2, 1/1.4) and two pressure spikes (x1.5 .. x4); T = p / (rho Rg)."""
    s = (n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG)
    rng = np.random.default_rng(seed)
    amp = np.geomspace(1e-3, 0.1, s[2])[None, None, :]
    Q = np.zeros((6, *s))
    Q[0] = 1.0 + amp * rng.uniform(-1, 1, s)
    Q[1:4] = 0.2 + amp * rng.uniform(-1, 1, (3, *s))
    Q[4] = (1.0 + amp * rng.uniform(-1, 1, s)) / 1.4
    for _ in range(2):
        a, b, c = [int(rng.integers(NG, k - NG)) for k in s]
        Q[4, a, b, c] *= float(rng.uniform(1.5, 4))
    Q[5] = Q[4] / (Q[0] * P.rg)
    return Q


def metrics_digest(m, J) -> str:
    """SHA-256 of the nine metrics and J as little-endian binary64."""
    h = hashlib.sha256()
    for a in (*m, J):
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def f64_digest(*arrays) -> str:
    """SHA-256 of the arrays as little-endian binary64, in order."""
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def _step_variants(module, P, Q, m, J, name, xyz=None):
    """RK3_STEPS steps of the time_step loop per STEP_VARIANTS entry from U = prim2c(Q) (xyz:
    the cell-centre coordinates of a finite-volume case)."""
    U0 = runtime.prim2c(module, P, Q)
    out = {}
    for label, kw in STEP_VARIANTS.items():
        U, Qs = runtime.rk3_steps(module, params_copy(P, **kw), U0, m, J, RK3_DT, RK3_STEPS, Q0=Q, xyz=xyz)
        out[f"{name}__steps_{label}_sha256"] = np.array(f64_digest(U, Qs))
    return out


def f32_digest(*arrays) -> str:
    """SHA-256 of the arrays as little-endian binary32, in order."""
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f4").tobytes())
    return h.hexdigest()


def _ref32(typed, P, Q, m, J, name, xyz):
    """The Float32 digests of one finite-difference case."""
    Q32, m32, J32 = (np.asarray(a, dtype=np.float32) for a in (Q, m, J))
    out = {f"{name}__rhs32_sha256": np.array(f32_digest(runtime.rhs(typed, P, Q32, m32, J32, typed=True))),
           f"{name}__metrics32_sha256": np.array(f32_digest(*runtime.metrics(
               typed, P, *(np.asarray(a, dtype=np.float32) for a in xyz), typed=True))),
           f"{name}__metrics32_readfort_sha256": np.array(f32_digest(*runtime.metrics(
               typed, P, *(np.asarray(a, dtype=np.float32) for a in xyz), typed=True, source="readfort")))}
    if runtime.is_reference_bcs(P):
        U0, Qf, Uf = runtime.state_and_ghosts(typed, P, Q32, typed=True)
        U, Qs = runtime.rk3_steps(typed, P, U0, m32, J32, RK3_DT, RK3_STEPS, Q0=Q32, typed=True)
        out[f"{name}__state32_sha256"] = np.array(f32_digest(U0, Qf, Uf, U, Qs))
        for label, kw in STEP_VARIANTS.items():  # the time_step loop in Float32
            U, Qs = runtime.rk3_steps(typed, params_copy(P, **kw), U0, m32, J32, RK3_DT, RK3_STEPS, Q0=Q32, typed=True)
            out[f"{name}__steps32_{label}_sha256"] = np.array(f32_digest(U, Qs))
    return out


def ghost_inputs():
    """Interior coordinates in millimetres (zero ghosts) of a curved 7 x 6 x 5 grid."""
    n = (7, 6, 5)
    s = (n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG)
    rng = np.random.default_rng(5)
    kk, jj, ii = np.meshgrid(*[np.arange(v, dtype=float) for v in s], indexing="ij")
    f = [ii + 0.1 * np.sin(jj), 1.3 * jj + 0.2 * np.cos(ii), 0.7 * kk + 0.05 * ii * jj / 40]
    I3 = (slice(NG, -NG),) * 3
    out = []
    for a in f:
        c = np.zeros(s)
        c[I3] = ((a + rng.uniform(-0.01, 0.01, s)) * 1000.0)[I3]
        out.append(c)
    return n, out


def _ghosts(module, typed):
    n, xyz = ghost_inputs()
    P = make_params(*n)
    out = {"ghosts__x": xyz[0], "ghosts__y": xyz[1], "ghosts__z": xyz[2]}
    for rule in ("readfort", "solver"):
        for label, mod, t in (("64", module, False), ("32", typed, True)):
            g = runtime.ghost_coordinates(mod, P, *xyz, rule=rule, typed=t)
            out[f"ghosts__{rule}{label}_sha256"] = np.array((f32_digest if t else f64_digest)(*g))
    return out


def _golden():
    spec = importlib.util.spec_from_file_location("make_golden", HERE / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _state_steps(module, P, Q, m, J, name):
    """For boundary.jl's own boundary set: U = prim2c(Q), then c2Prim and the ghost fill of a
    stage, and RK3_STEPS SSP-RK3 steps of dt = RK3_DT from (U, Q)."""
    U0, Qf, Uf = runtime.state_and_ghosts(module, P, Q)
    U, Qs = runtime.rk3_steps(module, P, U0, m, J, RK3_DT, RK3_STEPS, Q0=Q)
    return {f"{name}__U_prim2c": U0, f"{name}__Q_filled": Qf, f"{name}__U_filled": Uf,
            f"{name}__U_rk3": U, f"{name}__Q_rk3": Qs}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference source tree")
    a = ap.parse_args()
    ref = Path(a.ref)
    module = ROOT / "oracle" / "_ref" / "jl_kernels.py"
    corrected = ROOT / "oracle" / "_ref" / "jl_kernels_corrected.py"
    typed = ROOT / "oracle" / "_ref" / "jl_kernels_typed.py"
    module.parent.mkdir(parents=True, exist_ok=True)
    module.write_text(jl2py.translate_tree(ref))
    corrected.write_text(jl2py.translate_tree(ref, corrected=True))
    typed.write_text(jl2py.translate_tree(ref, typed=True))
    out = {"provenance": np.array(json.dumps({
        "translated": {f: hashlib.sha256((ref / f).read_bytes()).hexdigest()
                       for f in (*jl2py.FILES, "parse_mesh.jl", jl2py.READFORT)},
        "module_sha256": hashlib.sha256(module.read_bytes()).hexdigest(),
        "corrected_module_sha256": hashlib.sha256(corrected.read_bytes()).hexdigest(),
        "typed_module_sha256": hashlib.sha256(typed.read_bytes()).hexdigest(),
        "corrections": [c[-1] for c in jl2py.CORRECTIONS],
        "semantics": "every value binary64; Julia's literal powers x^2, x^3 as products, other powers by C pow",
        "rk3": {"dt": RK3_DT, "steps": RK3_STEPS}, "step_variants": STEP_VARIANTS}))}
    report = {}
    for f in sorted(HERE.glob("*.npz")):
        d = np.load(f, allow_pickle=True)
        if "rhs" not in d.files:  # RHS fixtures only
            continue
        meta = json.loads(str(d["meta"]))
        P = make_params(*meta["n"], **meta["params"])
        r = runtime.rhs(module, P, d["Q"], d["metrics"], d["J"])
        out[f"{f.stem}__rhs"] = r
        mr, Jr = runtime.metrics(module, P, d["x"], d["y"], d["z"])  # parse_mesh.jl:139-248
        out[f"{f.stem}__metrics_sha256"] = np.array(metrics_digest(mr, Jr))
        report[f.stem] = r
        if runtime.is_reference_bcs(P):
            out.update(_state_steps(module, P, d["Q"], d["metrics"], d["J"], f.stem))
        out.update(_ref32(typed, P, d["Q"], d["metrics"], d["J"], f.stem, (d["x"], d["y"], d["z"])))
    g = _golden()
    for name, spec in VISCOUS.items():
        n, params = spec["n"], dict(spec["params"])
        P = make_params(*n, **params)
        x, y, z = g.coords(n)
        Q = g.initial(P, n, spec["seed"], spec["spikes"], False, x, y, z)
        U = orc.prim2c(P, Q)
        orc.fill_ghosts(P, Q, U)
        m, J = runtime.metrics(module, P, x, y, z)  # the reference's own metrics (parse_mesh.jl:139-248)
        r = runtime.rhs(module, P, Q, m, J)
        meta = dict(n=list(n), params=params)
        out.update({f"{name}__Q": Q, f"{name}__metrics": m, f"{name}__J": J, f"{name}__rhs": r,
                    f"{name}__x": x, f"{name}__y": y, f"{name}__z": z,
                    f"{name}__metrics_sha256": np.array(metrics_digest(m, J)),
                    f"{name}__meta": np.array(json.dumps(meta))})
        report[name] = r
        if runtime.is_reference_bcs(P):
            out.update(_state_steps(module, P, Q, m, J, name))
            out.update(_step_variants(module, P, Q, m, J, name))
        out.update(_ref32(typed, P, Q, m, J, name, (x, y, z)))
        # the local time step (utils.jl:73-99) and the two filters (solver.jl:446-470)
        U = runtime.prim2c(module, P, Q)
        out[f"{name}__local_dt"] = runtime.local_dt(module, P, Q, m, J)
        for filt, label in ((1, "linear"), (2, "shock")):
            out[f"{name}__U_filter_{label}"] = runtime.filter_pass(module, params_copy(P, filter=filt), U, Q)
    for name, spec in FVM.items():
        n, params = spec["n"], {**FVM_COMMON, **spec["params"]}
        P = make_params(*n, **params)
        x, y, z = g.coords(n)
        Q = fvm_state(P, n, spec["seed"])
        U = orc.prim2c(P, Q)
        orc.fill_ghosts(P, Q, U)
        m, J = runtime.metrics(module, P, x, y, z)
        xyz = (x, y, z)
        out.update({f"{name}__Q": Q, f"{name}__x": x, f"{name}__y": y, f"{name}__z": z,
                    f"{name}__metrics_sha256": np.array(metrics_digest(m, J)),
                    f"{name}__meta": np.array(json.dumps(dict(n=list(n), params=params)))})
        for d, (fc, fw) in enumerate(zip(runtime.fvm_faces(corrected, P, Q, m, xyz),
                                         runtime.fvm_faces(module, P, Q, m, xyz))):
            out[f"{name}__F{d}"], out[f"{name}__F{d}_as_written"] = fc, fw
        r = runtime.rhs(corrected, P, Q, m, J, xyz)
        out[f"{name}__rhs_fvm"] = r
        report[name] = r
        if runtime.is_reference_bcs(P):
            Us, Qs = runtime.rk3_steps(corrected, P, runtime.prim2c(module, P, Q), m, J, RK3_DT, RK3_STEPS,
                                       Q0=Q, xyz=xyz)
            out[f"{name}__U_rk3_fvm"], out[f"{name}__Q_rk3_fvm"] = Us, Qs
            out.update(_step_variants(corrected, P, Q, m, J, name, xyz))
    out.update(_ghosts(module, typed))
    out["flat_plate_9x7x5_sha256"] = np.array(f32_digest(*runtime.flat_plate(typed, make_params(9, 7, 5), typed=True)))
    np.savez_compressed(HERE / "jl_reference_rhs.npz", **out)
    for name, r in report.items():
        print(name, "max |rhs|", float(np.abs(r[I]).max()))


if __name__ == "__main__":
    main()

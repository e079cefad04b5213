"""The oracle against the reference's own Julia kernels, translated mechanically into Python
(oracle/ref_jl/jl2py.py, run by oracle/ref_jl/runtime.py; CPU only).

tests/golden/jl_reference_rhs.npz holds the reference's finite-difference RHS, so computed
(tests/golden/make_jl_reference.py), on the golden fixtures' inputs and on five viscous
cases (two with the LES closures), and for the cases with boundary.jl's own boundary set its
prim2c, c2Prim with the ghost fill and two SSP-RK3 steps; and its finite-volume faces, RHS
and steps. The FP64 oracle must equal all of it bit for bit: the same
statements in the same order, in binary64 (the oracle is built without FMA contraction). With F3D_REFERENCE naming the reference tree,
the translation is regenerated and must reproduce the digest recorded with the fixture.
"""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from flame3d_mhd_gb300.abi import make_params
from oracle import oracle as orc
from oracle.ref_jl import jl2py
from oracle.ref_jl.runtime import JArray

ROOT = Path(__file__).resolve().parent.parent
FIX = ROOT / "tests" / "golden" / "jl_reference_rhs.npz"
NG = 4
I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))


def _cases():
    d = np.load(FIX, allow_pickle=True)
    names = sorted({k.split("__")[0] for k in d.files if k.endswith("__rhs")})
    return d, names


def _inputs(d, name):
    if f"{name}__Q" in d.files:
        meta = json.loads(str(d[f"{name}__meta"]))
        return meta, d[f"{name}__Q"], d[f"{name}__metrics"], d[f"{name}__J"]
    g = np.load(ROOT / "tests" / "golden" / f"{name}.npz", allow_pickle=True)
    return json.loads(str(g["meta"])), g["Q"], g["metrics"], g["J"]


@pytest.mark.parametrize("name", _cases()[1])
def test_oracle_equals_the_translated_reference(name):
    d, _ = _cases()
    meta, Q, m, J = _inputs(d, name)
    P = make_params(*meta["n"], **meta["params"])
    ro = orc.rhs(P, Q, list(m), J)
    ref = d[f"{name}__rhs"]
    assert np.abs(ref[I]).max() > 0
    assert np.array_equal(ro[I], ref[I]), float(np.abs(ro[I] - ref[I]).max())


def _state_cases():
    d, names = _cases()
    return [n for n in names if f"{n}__U_rk3" in d.files]


@pytest.mark.parametrize("name", _state_cases())
def test_oracle_state_ghosts_and_steps_equal_the_translated_reference(name):
    """prim2c, c2Prim with the ghost fill (boundary.jl's own boundary set, every cell including
    edges and corners) and two SSP-RK3 steps of the stage loop (solver.jl:416-444): bit for bit."""
    d, _ = _cases()
    meta, Q, m, J = _inputs(d, name)
    P = make_params(*meta["n"], **meta["params"])
    U = orc.prim2c(P, Q)
    assert np.array_equal(U, d[f"{name}__U_prim2c"])
    Qf, Uf = orc.c2prim(P, U), U.copy()
    orc.fill_ghosts(P, Qf, Uf)
    assert np.array_equal(Qf, d[f"{name}__Q_filled"]) and np.array_equal(Uf, d[f"{name}__U_filled"])
    rk = json.loads(str(d["provenance"]))["rk3"]
    Us, Un, Qs = U.copy(), np.zeros_like(U), np.array(Q, dtype=np.float64)
    orc.rk3(P, rk["steps"], rk["dt"], Us, Un, Qs, list(m), J)
    assert np.array_equal(Us, d[f"{name}__U_rk3"]) and np.array_equal(Qs, d[f"{name}__Q_rk3"])


@pytest.mark.parametrize("name", [n for n in _cases()[1] if f"{n}__local_dt" in _cases()[0].files])
def test_oracle_local_dt_and_filters_equal_the_translated_reference(name):
    """compute_dt (utils.jl:73-99) and one pass of the linear and of the shock-capturing filter
    (solver.jl:446-470, utils.jl:102-315): bit for bit."""
    from flame3d_mhd_gb300.cases import params_copy
    d, _ = _cases()
    meta, Q, m, J = _inputs(d, name)
    P = make_params(*meta["n"], **meta["params"])
    assert np.array_equal(orc.local_dt(P, Q, list(m), J), d[f"{name}__local_dt"])
    U = orc.prim2c(P, Q)
    for filt, label in ((1, "linear"), (2, "shock")):
        Uf, Un = U.copy(), np.zeros_like(U)
        orc.filter_pass(params_copy(P, filter=filt), Uf, Un, Q)
        ref = d[f"{name}__U_filter_{label}"]
        assert not np.array_equal(ref, U) and np.array_equal(Uf, ref), label


def _f64_digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", [n for n in _cases()[1] if f"{n}__steps_lts_sha256" in _cases()[0].files])
def test_oracle_time_step_loop_equals_the_translated_reference(name):
    """Two steps of the whole time_step loop (solver.jl:410-470) with local time stepping
    (compute_dt at the first stage of each step, div_LTS in every stage) and with either filter
    after every filtering_interval-th step, alone and together: U and Q bit for bit."""
    from flame3d_mhd_gb300.cases import params_copy
    d, _ = _cases()
    meta, Q, m, J = _inputs(d, name)
    P = make_params(*meta["n"], **meta["params"])
    prov = json.loads(str(d["provenance"]))
    rk = prov["rk3"]
    U0 = orc.prim2c(P, Q)
    for label, kw in prov["step_variants"].items():
        U, Un, Qs = U0.copy(), np.zeros_like(U0), np.array(Q, dtype=np.float64)
        orc.rk3(params_copy(P, **kw), rk["steps"], rk["dt"], U, Un, Qs, list(m), J)
        assert _f64_digest(U, Qs) == str(d[f"{name}__steps_{label}_sha256"]), label


def _digest(m, J):
    import hashlib
    h = hashlib.sha256()
    for a in (*m, J):
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", _cases()[1])
def test_oracle_metrics_equal_the_translated_reference(name):
    """The nine J^-1-scaled metrics and J of parse_mesh.jl:139-248 (CD6 inside, one-sided CD2
    in the outer three layers): bit for bit."""
    d, _ = _cases()
    meta = _inputs(d, name)[0]
    P = make_params(*meta["n"], **meta["params"])
    src = d if f"{name}__x" in d.files else np.load(ROOT / "tests" / "golden" / f"{name}.npz", allow_pickle=True)
    pre = f"{name}__" if src is d else ""
    m, J = orc.metrics(P, src[pre + "x"], src[pre + "y"], src[pre + "z"])
    assert _digest(m, J) == str(d[f"{name}__metrics_sha256"])
    # the metrics the RHS cases were computed from are these
    assert _digest(src[pre + "metrics"], src[pre + "J"]) == str(d[f"{name}__metrics_sha256"])


def test_fixture_covers_the_forms():
    d, names = _cases()
    forms = set()
    for name in names:
        p = _inputs(d, name)[0]["params"]
        forms.add((p.get("split_method", 0), p.get("character", 1), p.get("viscous", 0), p.get("les", 0)))
    assert {f[0] for f in forms} == {0, 1, 2, 3}  # SW, LF, VL, AUSM
    assert {f[1] for f in forms} == {0, 1} and {f[2] for f in forms} == {0, 1}
    assert {f[3] for f in forms} == {0, 1, 2}  # laminar, Smagorinsky, WALE


REF = Path(os.environ.get("F3D_REFERENCE", "")) if os.environ.get("F3D_REFERENCE") else None


@pytest.mark.skipif(REF is None or not (REF / "schemes.jl").exists(),
                    reason="F3D_REFERENCE does not name the reference tree")
def test_translation_reproduces_the_fixture_digest():
    import hashlib
    prov = json.loads(str(np.load(FIX, allow_pickle=True)["provenance"]))
    for f, h in prov["translated"].items():
        assert hashlib.sha256((REF / f).read_bytes()).hexdigest() == h, f
    assert hashlib.sha256(jl2py.translate_tree(REF).encode()).hexdigest() == prov["module_sha256"]
    assert hashlib.sha256(jl2py.translate_tree(REF, True).encode()).hexdigest() == prov["corrected_module_sha256"]
    assert hashlib.sha256(jl2py.translate_tree(REF, typed=True).encode()).hexdigest() == prov["typed_module_sha256"]


# ---- the reference's Float32 arithmetic (the REF32 form), from the typed translation
def _f32_digest(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f4").tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", [n for n in _cases()[1] if f"{n}__rhs32_sha256" in _cases()[0].files])
def test_oracle_float32_form_equals_the_typed_translation(name):
    """The oracle's Float32 restatement (the reference's own precision: Float32 arrays and
    arithmetic, WENO7 alphas in Float64 through WENOϵ1::Float64) against the reference's kernels
    evaluated with Julia's types: the RHS and, for boundary.jl's boundary set, prim2c, c2Prim
    with the ghost fill and two SSP-RK3 steps, bit for bit."""
    d, _ = _cases()
    meta, Q, m, J = _inputs(d, name)
    P = make_params(*meta["n"], **meta["params"])
    Q32, J32 = np.asarray(Q, dtype=np.float32), np.asarray(J, dtype=np.float32)
    m32 = [np.ascontiguousarray(a, dtype=np.float32) for a in m]
    assert _f32_digest(orc.rhs32(P, Q32, m32, J32)) == str(d[f"{name}__rhs32_sha256"])
    if f"{name}__state32_sha256" in d.files:
        rk = json.loads(str(d["provenance"]))["rk3"]
        U0 = orc.prim2c32(P, Q32)
        Qf, Uf = orc.c2prim32(P, U0), U0.copy()
        orc.fill_ghosts32(P, Qf, Uf)
        Us, Un, Qs = U0.copy(), np.zeros_like(U0), Q32.copy()
        orc.rk3_32(P, rk["steps"], np.float32(rk["dt"]), Us, Un, Qs, m32, J32)
        assert _f32_digest(U0, Qf, Uf, Us, Qs) == str(d[f"{name}__state32_sha256"])
        from flame3d_mhd_gb300.cases import params_copy
        for label, kw in json.loads(str(d["provenance"]))["step_variants"].items():  # LTS, filters
            Us, Un, Qs = U0.copy(), np.zeros_like(U0), Q32.copy()
            orc.rk3_32(params_copy(P, **kw), rk["steps"], np.float32(rk["dt"]), Us, Un, Qs, m32, J32)
            assert _f32_digest(Us, Qs) == str(d[f"{name}__steps32_{label}_sha256"]), label


@pytest.mark.parametrize("name", [n for n in _cases()[1] if f"{n}__metrics32_sha256" in _cases()[0].files])
def test_float32_set_up_metrics_equal_the_typed_translation(name):
    """meshgen.metrics_f32 (the host set-up of the Float32 form; the device's
    f3d_compute_metrics_f32 equals it bit for bit) against parse_mesh.jl:139-248 and
    readfort.jl:104-208 evaluated in their own types: Float32 coordinates and arrays, Float64
    (parse_mesh.jl: 1/60, 0.5, ...) or Float32 (readfort.jl) CD6 / CD2 coefficients, bit for bit."""
    from flame3d_mhd_gb300 import meshgen
    d, _ = _cases()
    src = d if f"{name}__x" in d.files else np.load(ROOT / "tests" / "golden" / f"{name}.npz", allow_pickle=True)
    pre = f"{name}__" if src is d else ""
    x, y, z = (np.asarray(src[pre + a], dtype=np.float32) for a in "xyz")
    m, J = meshgen.metrics_f32(x, y, z, coefficients="parse_mesh")
    assert _f32_digest(*m, J) == str(d[f"{name}__metrics32_sha256"])
    # readfort.jl:104-208, the same stencils with Float32 coefficients (1/60f0, 0.5f0, ...)
    m, J = meshgen.metrics_f32(x, y, z, coefficients="readfort")
    assert _f32_digest(*m, J) == str(d[f"{name}__metrics32_readfort_sha256"])


@pytest.mark.parametrize("rule", ["readfort", "solver"])
def test_ghost_coordinates_equal_the_translated_reference(tmp_path, rule):
    """grid.extend_ghosts (and, for readfort.jl, grid.mesh_from_ocfd reading a mesh file)
    against readfort.jl's generateXYZ (:34-99: reflections, edge completions, ./= 1000) and
    solver.jl's extrapolation, in binary64 and in Float32: bit for bit."""
    from flame3d_mhd_gb300 import grid
    d = np.load(FIX, allow_pickle=True)
    xyz = [d["ghosts__x"], d["ghosts__y"], d["ghosts__z"]]
    for dt, label, dig in ((np.float64, "64", _f64_digest), (np.float32, "32", _f32_digest)):
        g = grid.extend_ghosts(*[a.astype(dt) for a in xyz], dtype=dt, rule=rule)
        if rule == "readfort":
            g = tuple(a / dt(1000) for a in g)
        assert dig(*g) == str(d[f"ghosts__{rule}{label}_sha256"]), label
    if rule == "readfort":  # the mesh file's Float64 planes read into Float32 arrays
        nz, ny, nx = (v - 2 * NG for v in xyz[0].shape)
        path = str(tmp_path / "OCFD3d-Mesh.dat")
        grid.write_ocfd_mesh(path, *[a[NG:-NG, NG:-NG, NG:-NG] for a in xyz])
        g = grid.mesh_from_ocfd(path, nx, ny, nz)
        assert _f32_digest(*g) == str(d["ghosts__readfort32_sha256"])


def test_flat_plate_grid_equals_the_translated_reference():
    """meshgen.flat_plate_grid against parse_mesh.jl:38-136 evaluated with its types (Float32
    mapping of every cell, then the ghost reflections): bit for bit, with sinh taken in binary64
    and rounded to Float32 on both sides (Julia's own Float32 sinh may differ in the last bit)."""
    from flame3d_mhd_gb300 import meshgen
    d = np.load(FIX, allow_pickle=True)
    assert _f32_digest(*meshgen.flat_plate_grid(9, 7, 5)) == str(d["flat_plate_9x7x5_sha256"])


# ---- the translation rules on small pieces of Julia
def _py(src):
    return jl2py.translate(src).strip()


def test_rule_literals_and_products():
    assert jl2py.expr("-3V1+13V2") == "-3*V1+13*V2"
    assert jl2py.expr("1/12f0") == "1/12e0"
    assert jl2py.expr("x*1e-20 + 5f-2") == "x*1e-20 + 5e-2"
    assert jl2py.expr("(blockIdx().x-1i32)") == "(blockIdx().x-1)"
    assert jl2py.expr("2(a+b)") == "2*(a+b)"


def test_rule_powers_and_logic():
    assert jl2py.expr("u^2 + (a-b)^2 + x^3") == "_p2(u) + _p2((a-b)) + _p3(x)"
    assert jl2py.expr("F[i, j]^2") == "_p2(F[i, j])"
    assert jl2py.expr("T^1.5") == "T**1.5"
    assert jl2py.expr("a > b && !c || d != e") == "a > b  and   not c  or  d != e"


def test_rule_ternary_and_names():
    assert jl2py.expr("ifelse(a*b > 0, (abs(a) > abs(b)) ? b : a, zero(a))") == \
        "ifelse(a*b > 0,((b) if ((abs(a) > abs(b))) else (a)), zero(a))"
    assert jl2py.expr("∂ξ∂x") == "_u2202_ξ_u2202_x"


def test_rule_blocks_and_implicit_return():
    src = """
    # a comment
    @inline function f(a, b)
        ifelse(a > b, a, b)
    end
    function g(A, n)
        s::Float32 = 0.f0
        for m = 1:n
            @inbounds s += A[m] *
                           2
        end
        if s > 1; s = 1.f0; elseif s < 0
            s = 0
        else
            s = s
        end
        return s
    end
    """
    py = _py(src)
    ns = {"ifelse": lambda c, a, b: a if c else b}
    exec(py, ns)
    assert ns["f"](1, 2) == 2
    assert ns["g"](JArray(np.array([0.1, 0.2])), 2) == pytest.approx(0.6)  # 1-based A[m]
    assert ns["g"](JArray(np.array([1.0, 1.0])), 2) == 1.0


# ---- the finite-volume scheme (FVM.jl), from the translation with jl2py.CORRECTIONS applied
def _fvm_cases():
    d = np.load(FIX, allow_pickle=True)
    return sorted({k.split("__")[0] for k in d.files if k.endswith("__rhs_fvm")})


def _fvm_inputs(d, name):
    meta = json.loads(str(d[f"{name}__meta"]))
    P = make_params(*meta["n"], **meta["params"])
    x, y, z = (d[f"{name}__{a}"] for a in "xyz")
    m, J = orc.metrics(P, x, y, z)
    assert _digest(m, J) == str(d[f"{name}__metrics_sha256"])  # the reference's metrics
    return P, d[f"{name}__Q"], m, J, (x, y, z)


@pytest.mark.parametrize("name", _fvm_cases())
def test_oracle_fvm_faces_rhs_and_steps_equal_the_corrected_translation(name):
    """Face fluxes of the three directions, the RHS and (boundary.jl's boundary set) two SSP-RK3
    steps of the finite-volume scheme: bit for bit."""
    d = np.load(FIX, allow_pickle=True)
    P, Q, m, J, (x, y, z) = _fvm_inputs(d, name)
    eigen = int(P.scheme) == 1
    phi, U = orc.sensor(P, Q), orc.prim2c(P, Q)
    for dd in range(3):
        S = orc.metric_norm(P, m[3 * dd], m[3 * dd + 1], m[3 * dd + 2])
        F = orc.fvm_face_flux(P, dd, eigen, phi, S, Q, U, x, y, z)
        assert np.array_equal(F, d[f"{name}__F{dd}"]), (dd, float(np.abs(F - d[f"{name}__F{dd}"]).max()))
    orc.set_coordinates(x, y, z)
    try:
        r = orc.rhs(P, Q, list(m), J)
        assert np.abs(r[I]).max() > 0 and np.array_equal(r[I], d[f"{name}__rhs_fvm"][I])
        if f"{name}__U_rk3_fvm" in d.files:
            rk = json.loads(str(d["provenance"]))["rk3"]
            Us, Un, Qs = U.copy(), np.zeros_like(U), Q.copy()
            orc.rk3(P, rk["steps"], rk["dt"], Us, Un, Qs, list(m), J)
            assert np.array_equal(Us, d[f"{name}__U_rk3_fvm"]) and np.array_equal(Qs, d[f"{name}__Q_rk3_fvm"])
    finally:
        orc.set_coordinates(None)


@pytest.mark.parametrize("name", [n for n in _fvm_cases() if f"{n}__steps_lts_sha256" in np.load(FIX).files])
def test_oracle_fvm_time_step_loop_equals_the_corrected_translation(name):
    """Two steps of the time_step loop on the finite-volume scheme with local time stepping
    and/or either filter: U and Q bit for bit."""
    from flame3d_mhd_gb300.cases import params_copy
    d = np.load(FIX, allow_pickle=True)
    P, Q, m, J, (x, y, z) = _fvm_inputs(d, name)
    prov = json.loads(str(d["provenance"]))
    rk = prov["rk3"]
    U0 = orc.prim2c(P, Q)
    orc.set_coordinates(x, y, z)
    try:
        for label, kw in prov["step_variants"].items():
            U, Un, Qs = U0.copy(), np.zeros_like(U0), np.array(Q, dtype=np.float64)
            orc.rk3(params_copy(P, **kw), rk["steps"], rk["dt"], U, Un, Qs, list(m), J)
            assert _f64_digest(U, Qs) == str(d[f"{name}__steps_{label}_sha256"]), label
    finally:
        orc.set_coordinates(None)


def test_fvm_cases_cover_the_branches_and_forms():
    d = np.load(FIX, allow_pickle=True)
    forms, seen = set(), {1: set(), 2: set()}
    for name in _fvm_cases():
        P, Q, m, J, xyz = _fvm_inputs(d, name)
        forms.add((int(P.scheme), int(P.viscous)))
        orc.set_coordinates(*xyz)
        try:
            _, br = orc.rhs(P, Q, list(m), J, with_branches=True)
        finally:
            orc.set_coordinates(None)
        seen[int(P.scheme)] |= set(np.unique(np.concatenate([b.ravel() for b in br])).tolist())
    assert forms == {(1, 0), (1, 1), (2, 0), (2, 1)}
    assert seen[1] == seen[2] == {0, 1, 2, 3}  # linear, WENO7, WENO5, minmod faces


def test_fvm_defects_change_only_the_faces_they_reach():
    """The as-written translation differs from the corrected one exactly where the two defects
    of FVM.jl act: the WENO5 faces of the Roe-characteristic reconstruction (the overwritten
    kinetic energy) and the y and z faces of the component-wise one (states stored as fluxes)."""
    d = np.load(FIX, allow_pickle=True)
    for name in _fvm_cases():
        P, Q, m, J, (x, y, z) = _fvm_inputs(d, name)
        eigen = int(P.scheme) == 1
        phi, U = orc.sensor(P, Q), orc.prim2c(P, Q)
        for dd in range(3):
            Fc, Fw = d[f"{name}__F{dd}"], d[f"{name}__F{dd}_as_written"]
            differs = np.any(Fc != Fw, axis=0)
            if eigen:
                S = orc.metric_norm(P, m[3 * dd], m[3 * dd + 1], m[3 * dd + 2])
                _, br = orc.fvm_face_flux(P, dd, True, phi, S, Q, U, x, y, z, with_branch=True)
                assert np.array_equal(differs, br == 2), (name, dd)
            else:
                assert differs.all() if dd else not differs.any(), (name, dd)


def test_rule_typed_literals_and_locals():
    """Julia's types kept: Float32 literals, Float64 literals, typed locals converting on every
    assignment (x op= e included), typed temporaries."""
    assert jl2py.expr("1/12f0 + WENOϵ1*1e-20 - 2x + 0.5", typed=True) == "1/_f32(12e0) + WENOϵ1*_f64(1e-20) - 2*x + _f64(0.5)"
    assert jl2py.expr("MMatrix{5, 5, Float32, 25}(undef)", typed=True) == "_mat(5, 5, 32)"
    # Int / Int is Float64, unless the quotient continues a product or is raised to a power
    assert jl2py.expr("1/60*(f[7]-f[1])", typed=True) == "_f64(1/60)*(f[7]-f[1])"
    assert jl2py.expr("a*3/4", typed=True) == "a*3/4"
    assert jl2py.expr("1/2^k", typed=True) == "1/2**k"
    py = jl2py.translate("""
    function g(A, n)
        s::Float32 = 0.f0
        t = 0.f0
        for m = 1:n
            s += A[m] * 0.1
            t += A[m] * 0.1
        end
        return s, t
    end
    """, typed=True)
    assert "s = _f32(s + (A[m] * _f64(0.1)))" in py and "t += A[m] * _f64(0.1)" in py
    ns = {"_f32": np.float32, "_f64": np.float64}
    exec(py, ns)
    s_, t_ = ns["g"](JArray(np.array([1.0, 2.0], dtype=np.float32)), 2)
    assert type(s_) is np.float32 and type(t_) is np.float64  # t is Float64 after t += Float64, as in Julia


def test_rule_loops_and_ranges():
    """Loops over several variables and over named ranges, range assignments."""
    py = jl2py.translate("""
    function f(A)
        I_in = 2 : 3
        for k in I_in, j = 1:2
            A[j, k] = j + 10k
        end
    end
    """)
    assert "I_in = range(2, (3) + 1)" in py and "for k in I_in:" in py and "for j in range(1, (2) + 1):" in py
    ns = {}
    exec(py, ns)
    A = JArray(np.zeros((3, 2)))
    ns["f"](A)
    assert A.a.tolist() == [[0, 0], [21, 22], [31, 32]]


def test_rule_corrections_are_exact():
    """A correction applies only with its stated number of matches: a changed reference
    source fails loudly rather than being patched in part."""
    src = "function Eigen_reconstruct_i()\n    v2 = -1.0f0*V3L + 1\n    x = α2L*v2 + 1\nend\n" \
          "function Conser_reconstruct_i()\nend\nfunction Conser_reconstruct_j()\n" \
          "    Fy[1] = UR_final_1#flux_temp[1] * Area\nend\n"
    with pytest.raises(ValueError, match="matched 1 times, expected 6"):
        jl2py.apply_corrections("FVM.jl", src)
    assert jl2py.apply_corrections("split.jl", src) == src  # other files untouched


@pytest.mark.skipif(REF is None or not (REF / "schemes.jl").exists(),
                    reason="F3D_REFERENCE does not name the reference tree")
@pytest.mark.parametrize("seed", range(8))
def test_random_configurations_against_the_translation(tmp_path, seed):
    """Random split, reconstruction, thresholds, viscosity, LES, boundary set, grid and state
    (some near vacuum or with strong jumps): the FP64 RHS and the Float32 RHS equal the
    translated reference's bit for bit (NaN where it has NaN), and so does one SSP-RK3 step
    with the reference's boundary set."""
    import importlib.util
    from flame3d_mhd_gb300.abi import BC_PERIODIC
    from oracle.ref_jl import runtime
    mod, typed = tmp_path / "jl.py", tmp_path / "jl_typed.py"
    mod.write_text(jl2py.translate_tree(REF))
    typed.write_text(jl2py.translate_tree(REF, typed=True))
    spec = importlib.util.spec_from_file_location("make_golden", ROOT / "tests" / "golden" / "make_golden.py")
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    rng = np.random.default_rng(1000 + seed)
    th = [(0.02, 0.1, 0.4), (0.05, 1.0, 10.0), (0.0, 0.0, 1e30), (0.0, 1e30, 1e30), (0.0, 0.0, 0.0)][seed % 5]
    n = tuple(int(v) for v in rng.integers(5, 8, 3))
    visc = seed % 2
    kw = dict(split_method=seed % 4, character=(seed // 2) % 2, viscous=visc, les=(seed // 4) % 3 if visc else 0,
              phi1=th[0], phi2=th[1], phi3=th[2], rg=1.0, c_s=1e-2, t_s=1.0)
    if seed % 3 == 2:
        kw["bc"] = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(*n, **kw)
    x, y, z = g.coords(n)
    Q = g.initial(P, n, seed, int(rng.integers(0, 8)), False, x, y, z)
    if seed % 4 == 3:  # near vacuum and strong jumps
        Q[0] *= np.exp(rng.uniform(-4, 1, Q[0].shape))
        Q[4] *= np.exp(rng.uniform(-4, 2, Q[4].shape))
        Q[5] = Q[4] / (Q[0] * P.rg)
    U = orc.prim2c(P, Q)
    orc.fill_ghosts(P, Q, U)
    m, J = orc.metrics(P, x, y, z)
    m = np.stack(m)
    assert np.array_equal(runtime.rhs(mod, P, Q, m, J)[I], orc.rhs(P, Q, list(m), J)[I], equal_nan=True)
    Q32, m32, J32 = Q.astype(np.float32), m.astype(np.float32), J.astype(np.float32)
    assert np.array_equal(runtime.rhs(typed, P, Q32, m32, J32, typed=True)[I],
                          orc.rhs32(P, Q32, list(m32), J32)[I], equal_nan=True)
    if runtime.is_reference_bcs(P):
        Us, Qs = runtime.rk3_steps(mod, P, U, m, J, 1e-4, 1, Q0=Q)
        Uo, Un, Qo = U.copy(), np.zeros_like(U), Q.copy()
        orc.rk3(P, 1, 1e-4, Uo, Un, Qo, list(m), J)
        assert np.array_equal(Us, Uo, equal_nan=True) and np.array_equal(Qs, Qo, equal_nan=True)


@pytest.mark.skipif(REF is None or not (REF / "FVM.jl").exists(),
                    reason="F3D_REFERENCE does not name the reference tree")
@pytest.mark.parametrize("seed", range(4))
def test_random_fvm_configurations_against_the_corrected_translation(tmp_path, seed):
    """Random finite-volume configurations (reconstruction, viscosity, boundary set, noise
    growing along x, pressure spikes): the face fluxes and the RHS equal the corrected
    translation's bit for bit, and with the reference's boundary set so does one SSP-RK3 step,
    plain, with local time stepping and with the shock-capturing filter."""
    import importlib.util
    from flame3d_mhd_gb300.abi import BC_PERIODIC
    from flame3d_mhd_gb300.cases import params_copy
    from oracle.ref_jl import runtime
    mod = tmp_path / "jl_corrected.py"
    mod.write_text(jl2py.translate_tree(REF, corrected=True))
    spec = importlib.util.spec_from_file_location("make_golden", ROOT / "tests" / "golden" / "make_golden.py")
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    rng = np.random.default_rng(2000 + seed)
    n = tuple(int(v) for v in rng.integers(5, 8, 3))
    kw = dict(scheme=1 + seed % 2, viscous=(seed // 2) % 2, phi1=0.02, phi2=0.1, phi3=0.4, rg=1.0, c_s=1e-2, t_s=1.0)
    if seed == 3:
        kw["bc"] = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(*n, **kw)
    x, y, z = g.coords(n)
    s = (n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG)
    amp = np.geomspace(1e-3, 0.1, s[2])[None, None, :]
    Q = np.zeros((6, *s))
    Q[0] = 1.0 + amp * rng.uniform(-1, 1, s)
    Q[1:4] = rng.uniform(-0.3, 0.3, (3, 1, 1, 1)) + amp * rng.uniform(-1, 1, (3, *s))
    Q[4] = (1.0 + amp * rng.uniform(-1, 1, s)) / 1.4
    for _ in range(2):
        a, b, c = [int(rng.integers(NG, k - NG)) for k in s]
        Q[4, a, b, c] *= float(rng.uniform(1.5, 6))
    Q[5] = Q[4] / (Q[0] * P.rg)
    U = orc.prim2c(P, Q)
    orc.fill_ghosts(P, Q, U)
    m, J = orc.metrics(P, x, y, z)
    m = np.stack(m)
    phi, Uq = orc.sensor(P, Q), orc.prim2c(P, Q)
    for d, F in enumerate(runtime.fvm_faces(mod, P, Q, m, (x, y, z))):
        S = orc.metric_norm(P, m[3 * d], m[3 * d + 1], m[3 * d + 2])
        assert np.array_equal(F, orc.fvm_face_flux(P, d, int(P.scheme) == 1, phi, S, Q, Uq, x, y, z), equal_nan=True)
    r = runtime.rhs(mod, P, Q, m, J, (x, y, z))
    orc.set_coordinates(x, y, z)
    try:
        assert np.array_equal(r[I], orc.rhs(P, Q, list(m), J)[I], equal_nan=True)
        if runtime.is_reference_bcs(P):
            for v in ({}, dict(lts=1, lts_cfl=0.3), dict(filter=2, filter_interval=1, filter_rth=1e-5)):
                Pv = params_copy(P, **v)
                Us, Qs = runtime.rk3_steps(mod, Pv, U, m, J, 1e-4, 1, Q0=Q, xyz=(x, y, z))
                Uo, Un, Qo = U.copy(), np.zeros_like(U), Q.copy()
                orc.rk3(Pv, 1, 1e-4, Uo, Un, Qo, list(m), J)
                assert np.array_equal(Us, Uo, equal_nan=True) and np.array_equal(Qs, Qo, equal_nan=True), v
    finally:
        orc.set_coordinates(None)

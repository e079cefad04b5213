"""The Julia `ccall` declarations of INTEGRATION.md against the C prototypes of
include/flame3d_gpu.h (CPU only; Julia itself is not installed).

Every `ccall((:f3d_name, LIB), Ret, (ArgTypes...), args...)` must name an exported function,
with as many arguments as its prototype and, position by position, the same kind of
argument: Cint for int, Float64 for double, Float32 for float, Clonglong for long long, and
a pointer type (Ptr, CuPtr, Ref, Cstring) for a pointer, with CuPtr{Float64} / CuPtr{Float32}
only where the C parameter points to double / float. The call's argument list must have as
many entries as its type tuple. A swapped int and double would pass the C compiler of the
binding (Julia) unnoticed and only work by the accident of the calling convention.
"""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _balanced(s: str, i: int) -> int:
    """Index just past the bracket group opening at s[i]."""
    depth = 0
    pairs = {"(": ")", "{": "}", "[": "]"}
    stack = []
    for j in range(i, len(s)):
        c = s[j]
        if c in pairs:
            stack.append(pairs[c])
            depth += 1
        elif stack and c == stack[-1]:
            stack.pop()
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced")


def _split_top(s: str) -> list:
    out, depth, cur = [], 0, ""
    for c in s:
        if c in "({[":
            depth += 1
        elif c in ")}]":
            depth -= 1
        if c == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += c
    if cur.strip():
        out.append(cur.strip())
    return out


def c_prototypes() -> dict:
    text = (ROOT / "include" / "flame3d_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"(?:^|\n)\s*(?:const\s+)?(int|char\s*\*|const\s+char\s*\*)\s*(f3d_\w+)\s*\(", text):
        name = m.group(2)
        start = text.index("(", m.end() - 1)
        params = text[start + 1:_balanced(text, start) - 1]
        protos[name] = [] if params.strip() in ("", "void") else _split_top(params)
    return protos


def c_kind(param: str) -> str:
    p = " ".join(param.split())
    if "*" in p or "[" in p or p.startswith("f3d_stream"):
        if re.search(r"\bdouble\b", p) and p.count("*") + p.count("[") == 1:
            return "ptr:double"
        if re.search(r"\bfloat\b", p) and p.count("*") + p.count("[") == 1:
            return "ptr:float"
        return "ptr"
    if re.search(r"\blong long\b", p):
        return "longlong"
    if re.search(r"\bdouble\b", p):
        return "double"
    if re.search(r"\bfloat\b", p):
        return "float"
    if re.search(r"\bint\b", p):
        return "int"
    raise ValueError(f"unclassified C parameter: {param}")


def julia_kind(t: str) -> str:
    t = t.strip()
    scalars = {"Cint": "int", "Int32": "int", "Float64": "double", "Cdouble": "double", "Float32": "float",
               "Cfloat": "float", "Clonglong": "longlong", "Int64": "longlong"}
    if t in scalars:
        return scalars[t]
    if t == "CuPtr{Float64}":
        return "ptr:double"
    if t == "CuPtr{Float32}":
        return "ptr:float"
    if t.startswith(("Ptr{", "Ref{", "CuPtr{")) or t == "Cstring":
        return "ptr"
    raise ValueError(f"unclassified Julia type: {t}")


def julia_ccalls() -> list:
    text = (ROOT / "INTEGRATION.md").read_text()
    calls = []
    for m in re.finditer(r"ccall\(\(:(f3d_\w+),\s*LIB\)", text):
        start = m.start() + len("ccall")
        body = text[start + 1:_balanced(text, start) - 1]
        parts = _split_top(body)
        # parts: (:name, LIB), Ret, (types...), args...
        types = parts[2]
        assert types.startswith("(") and types.endswith(")"), (m.group(1), types)
        tlist = _split_top(types[1:-1])
        calls.append((m.group(1), parts[1], tlist, parts[3:]))
    return calls


def test_header_parses():
    protos = c_prototypes()
    assert "f3d_rk3_steps" in protos and len(protos["f3d_rk3_steps"]) == 7
    assert c_kind(protos["f3d_rk3_steps"][1]) == "int" and c_kind(protos["f3d_rk3_steps"][2]) == "double"


def test_every_ccall_matches_its_prototype():
    protos = c_prototypes()
    calls = julia_ccalls()
    assert len(calls) >= 15
    for name, ret, tlist, args in calls:
        assert name in protos, f"{name} is not declared in include/flame3d_gpu.h"
        cparams = protos[name]
        assert len(tlist) == len(cparams), f"{name}: {len(tlist)} Julia types, {len(cparams)} C parameters"
        assert len(args) == len(tlist), f"{name}: {len(args)} arguments for {len(tlist)} types"
        for k, (jt, cp) in enumerate(zip(tlist, cparams)):
            jk, ck = julia_kind(jt), c_kind(cp)
            if jk == "ptr" or ck == "ptr":
                ok = jk.startswith("ptr") and ck.startswith("ptr")
            else:
                ok = jk == ck
            assert ok, f"{name} argument {k + 1}: Julia {jt} for C '{cp}'"
        assert ret in ("Cint", "Cstring"), f"{name}: return type {ret}"


def test_the_checker_catches_a_swap():
    """The swapped (Float64, Cint) of an earlier f3d_rk3_steps declaration is rejected."""
    protos = c_prototypes()
    cparams = protos["f3d_rk3_steps"]
    bad = ["Ptr{Cvoid}", "Float64", "Cint", "CuPtr{Float64}", "CuPtr{Float64}", "CuPtr{Float64}", "Ptr{Cvoid}"]
    kinds = [(julia_kind(j), c_kind(c)) for j, c in zip(bad, cparams)]
    assert any(not (a.startswith("ptr") and b.startswith("ptr")) and a != b for a, b in kinds)

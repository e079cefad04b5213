"""Mechanical translation of the reference's Julia GPU kernels into Python (test infrastructure).

The reference's hot path is Julia (CUDA.jl kernels) and no Julia is available, so the oracle
(oracle/f3d_oracle.hpp) is a restatement written by hand. To check that restatement against
the reference's own source, this script translates the kernel files (split.jl, schemes.jl,
viscous.jl, div.jl, utils.jl, boundary.jl, FVM.jl) and the metric computations of two
scripts (parse_mesh.jl, SCU-benchmark/readfort.jl) statement by statement, with fixed rules
and no hand edits:

- comments dropped; a line ending in an operator, a comma or an open bracket continues;
  ';' separates statements;
- `function f(args)` .. `end`, `if` / `elseif` / `else`, `for v = a:b` become Python blocks
  (`begin` .. `end` adds none); a bare expression ending a function body is returned, as
  Julia returns it;
- `@inbounds`, `@fastmath`, `@inline`, `@view` and type annotations (`x::Float32 = ...`) are
  dropped (a view reads what its slice reads);
- literals: `12f0` -> `12e0`, `1i32` -> `1`, implicit products `547V1` -> `547*V1`;
- `x^2` / `x^3` -> `_p2(x)` / `_p3(x)` (products, as Julia's literal powers), other `^` -> `**`,
  `&&` / `||` / `!` -> `and` / `or` / `not`, `c ? a : b` -> `(a if c else b)`,
  `x .= v` -> `x._fill(v)`, `MMatrix{n, m, ...}(undef)` / `MVector{n, ...}(undef)` /
  `SVector{...}(values)` -> 1-based arrays, `@cuda <keywords> f(args)` -> `_cuda(f, args)` (a launch the runtime runs over the
  grid), `CUDA.eps(Float32)` -> 2^-23, `÷` -> `//`, a character Julia allows in names and
  Python does not (the ∂ of ∂ξ∂x) -> `_u2202_`;
- array indexing is left as written: the runtime (runtime.py) passes arrays that take
  Julia's 1-based, column-major subscripts; in the scripts, `a:b` and `:` subscripts become
  slices, loops over several variables nest, `@.` broadcasts run elementwise.

In this FP64 reading every value is a binary64 scalar; the reference's Float32
annotations and f0 literals select the element type only, so the result is the reference's
algorithm evaluated in FP64 in the reference's own operation order, the form the FP64 oracle
restates. The generated module is written next to the compiled reference program
(oracle/_ref/, not tracked).

`translate_tree(root, typed=True)` keeps Julia's element types instead, for an evaluation of
the reference's own precision in NumPy scalars: `12f0` -> `_f32(12e0)` (Float32), `1e-20` /
`0.5` -> `_f64(...)` (Float64), an Int / Int quotient -> `_f64(a/b)`, other integer literals
left as they are (Python ints take the other operand's type, as Julia's Int does), `zeros(
Float32, ...)` -> Float32 arrays, a local declared `x::Float32` / `x::Float64`
converted at every assignment to it (`x op= e` included), `MMatrix` / `MVector` temporaries of
their element type. The runtime then supplies Float32 arrays and run.jl's Float32 constants.

`translate_tree(root, corrected=True)` first applies CORRECTIONS, two defects of FVM.jl
repaired by exact text substitutions, each of which must match the stated number of times;
everything else is translated as written.

    python -m oracle.ref_jl.jl2py <reference root> [out.py] [--corrected] [--typed]
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

FILES = ("split.jl", "schemes.jl", "viscous.jl", "div.jl", "utils.jl", "boundary.jl", "FVM.jl")

# (file, region from / to (text markers, None = file start / end), pattern, replacement,
#  matches, why)
CORRECTIONS = (
    ("FVM.jl", None, "function Conser_reconstruct_i", r"\bv2 = -1\.0f0\*V3([LR])", r"v2c = -1.0f0*V3\1", 6,
     "Eigen_reconstruct_i/j/k, WENO5 branch (FVM.jl:178, 198, 399, 414, 615, 630): the candidate v2 "
     "reuses the name of the Roe-averaged kinetic energy v2 (FVM.jl:73, 310, 526), a local of the "
     "enclosing function, so the loop body assigns that variable and the right-eigenvector row of "
     "field 2 (rn5 = v2, FVM.jl:211, 426, 642) reads the candidate on WENO5 faces"),
    ("FVM.jl", None, "function Conser_reconstruct_i", r"α2([LR])\*v2 \+", r"α2\1*v2c +", 6,
     "the renamed candidate's uses (FVM.jl:181, 201, 401, 416, 617, 632)"),
    ("FVM.jl", "function Conser_reconstruct_j", None, r"= U[LR]_final_\d#(flux_temp\[\d\] \* Area)", r"= \1", 10,
     "Conser_reconstruct_j/k (FVM.jl:1037-1041, 1215-1219) store the reconstructed states, the "
     "flux flux_temp[n] * Area commented out after them"),
)


def apply_corrections(name: str, src: str) -> str:
    """src with every correction of file `name` applied; a count that differs raises."""
    for f, a, b, pat, rep, count, _ in CORRECTIONS:
        if f != name:
            continue
        i0 = src.index(a) if a else 0
        i1 = src.index(b) if b else len(src)
        region, n = re.subn(pat, rep, src[i0:i1])
        if n != count:
            raise ValueError(f"{name}: {pat!r} matched {n} times, expected {count}")
        src = src[:i0] + region + src[i1:]
    return src

_OPEN = "([{"
_CLOSE = ")]}"


def _depth_delta(s: str) -> int:
    d = 0
    for ch in s:
        if ch in _OPEN:
            d += 1
        elif ch in _CLOSE:
            d -= 1
    return d


def _strip_comment(line: str) -> str:
    out, in_str = [], False
    for ch in line:
        if ch == '"':
            in_str = not in_str
        if ch == "#" and not in_str:
            break
        out.append(ch)
    return "".join(out).rstrip()


def logical_lines(src: str) -> list[str]:
    """Comment-free statements: continuation lines joined, ';'-separated statements split."""
    phys = [_strip_comment(l) for l in src.splitlines()]
    joined, buf, depth = [], "", 0
    cont_end = ("+", "-", "*", "/", ",", "(", "[", "=", "&&", "||", "?", ":", "<", ">", "^")
    for l in phys:
        if not l.strip():
            if buf and depth > 0:
                continue
            if buf:
                joined.append(buf)
                buf = ""
            continue
        buf = (buf + " " + l.strip()) if buf else l
        depth += _depth_delta(l)
        if depth > 0 or buf.rstrip().endswith(cont_end):
            continue
        joined.append(buf)
        buf, depth = "", 0
    if buf:
        joined.append(buf)
    out = []
    for l in joined:
        parts, cur, d = [], "", 0
        for ch in l:
            if ch in _OPEN:
                d += 1
            elif ch in _CLOSE:
                d -= 1
            if ch == ";" and d == 0:
                parts.append(cur)
                cur = ""
            else:
                cur += ch
        parts.append(cur)
        out.extend(p for p in parts if p.strip())
    return out


_NUM = r"(?<![\w.])(\d+\.\d*|\.\d+|\d+)"


def _ternary(s: str) -> str:
    """Rewrite the innermost `cond ? a : b` (at one bracket depth) until none is left."""
    while "?" in s:
        q = s.index("?")
        # the bracket depth at q, and the span of the enclosing group or argument
        depth = 0
        start = 0
        for i in range(q - 1, -1, -1):
            ch = s[i]
            if ch in _CLOSE:
                depth += 1
            elif ch in _OPEN:
                if depth == 0:
                    start = i + 1
                    break
                depth -= 1
            elif ch == "," and depth == 0:
                start = i + 1
                break
        depth = 0
        colon = end = None
        for i in range(q + 1, len(s)):
            ch = s[i]
            if ch in _OPEN:
                depth += 1
            elif ch in _CLOSE:
                if depth == 0:
                    end = i
                    break
                depth -= 1
            elif ch == ":" and depth == 0 and colon is None:
                colon = i
            elif ch == "," and depth == 0 and colon is not None:
                end = i
                break
        if end is None:
            end = len(s)
        if colon is None:
            raise ValueError(f"ternary without ':' in {s!r}")
        cond, a, b = s[start:q].strip(), s[q + 1:colon].strip(), s[colon + 1:end].strip()
        s = s[:start] + f"(({a}) if ({cond}) else ({b}))" + s[end:]
    return s


def _literal_powers(s: str) -> str:
    """x^2 -> _p2(x), x^3 -> _p3(x): Julia evaluates a literal integer power as products
    (Base.literal_pow: x*x, x*x*x), which a libm pow does not always round alike."""
    while True:
        m = re.search(r"\*\*([23])(?![\d.eE])", s)
        if not m:
            return s
        end = m.start()
        i = end - 1
        if s[i] in ")]":
            depth = 0
            while i >= 0:
                if s[i] in ")]":
                    depth += 1
                elif s[i] in "([":
                    depth -= 1
                    if depth == 0:
                        break
                i -= 1
            i -= 1
            while i >= 0 and (s[i].isalnum() or s[i] == "_" or ord(s[i]) > 127):  # a call's or an array's name
                i -= 1
        else:
            while i >= 0 and (s[i].isalnum() or s[i] in "_." or ord(s[i]) > 127):
                i -= 1
        start = i + 1
        s = s[:start] + f"_p{m.group(1)}({s[start:end]})" + s[m.end():]


def _ranges_in_brackets(s: str) -> str:
    """Inside [...] subscripts: `a:b` -> `_r(a, b)` and a bare `:` -> `_all` (Julia slices)."""
    out, i = [], 0
    while i < len(s):
        ch = s[i]
        if ch == "[" and i > 0 and (s[i - 1].isalnum() or s[i - 1] in "_]" or ord(s[i - 1]) > 127):
            depth, j = 0, i
            while j < len(s):
                if s[j] in "([{":
                    depth += 1
                elif s[j] in ")]}":
                    depth -= 1
                    if depth == 0:
                        break
                j += 1
            inner = _ranges_in_brackets(s[i + 1:j])
            parts, cur, d = [], "", 0
            for c in inner:
                if c in "([{":
                    d += 1
                elif c in ")]}":
                    d -= 1
                if c == "," and d == 0:
                    parts.append(cur)
                    cur = ""
                else:
                    cur += c
            parts.append(cur)
            conv = []
            for part in parts:
                t, d, colon = part, 0, None
                for k, c in enumerate(t):
                    if c in "([{":
                        d += 1
                    elif c in ")]}":
                        d -= 1
                    elif c == ":" and d == 0:
                        colon = k
                        break
                if colon is None:
                    conv.append(t)
                elif not t.strip() or t.strip() == ":":
                    conv.append("_all")
                else:
                    conv.append(f"_r({t[:colon].strip()}, {t[colon + 1:].strip()})")
            out.append("[" + ", ".join(c.strip() for c in conv) + "]")
            i = j + 1
            continue
        out.append(ch)
        i += 1
    return "".join(out)


def _typed_literal(m) -> str:
    num, f32 = m.group(1), m.group(2)
    if f32 is not None:
        return f"_f32({num}e{f32})"
    return f"_f64({num})" if re.search(r"[.eE]", num) else num


def expr(s: str, typed: bool = False) -> str:
    s = s.replace("CUDA.eps(Float32)", "_eps32()")
    if typed:
        s = re.sub(r"\bzeros\(\s*Float(32|64)\s*,", r"_zerosT(\1,", s)
    s = re.sub(r"\bzeros\(\s*Float(32|64)\s*,", "_zeros(", s)
    if ":" in s and "[" in s:
        s = _ranges_in_brackets(s)
    if typed:  # temporaries of the stated element type
        s = re.sub(r"MMatrix\{\s*([^,}]+)\s*,\s*([^,}]+)\s*,\s*Float(32|64)[^}]*\}\s*\(\s*undef\s*\)",
                   r"_mat(\1, \2, \3)", s)
        s = re.sub(r"MVector\{\s*([^,}]+)\s*,\s*Float(32|64)[^}]*\}\s*\(\s*undef\s*\)", r"_mat(\1, None, \2)", s)
    s = re.sub(r"MMatrix\{\s*([^,}]+)\s*,\s*([^,}]+)\s*,[^}]*\}\s*\(\s*undef\s*\)", r"_mat(\1, \2)", s)
    s = re.sub(r"MVector\{\s*([^,}]+)\s*,[^}]*\}\s*\(\s*undef\s*\)", r"_mat(\1)", s)
    s = re.sub(r"SVector\{[^}]*\}\s*\(", "_vec(", s)
    if typed:  # Int / Int is a Float64 quotient (1/60 -> _f64(1/60)); a quotient that continues a
        # product (a*3/4 is (a*3)/4) or is raised to a power (1/2^k) is left as it is
        s = re.sub(r"(?<![\w.*/^])(?<![*/^] )(\d+)\s*/\s*(\d+)(?![\w.^])(?! *\^)", r"_f64(\1/\2)", s)
    if typed:  # Float32 literals (12f0) -> _f32(12e0), Float64 ones (1e-20, 0.5) -> _f64(...)
        s = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|\d+(?:[eE][-+]?\d+)?)"
                   r"(?:f(-?\d+))?(?![\w.])", _typed_literal, s)
    s = re.sub(r"(\d+\.\d*|\.\d+|\d+)f(-?\d+)", r"\1e\2", s)          # Float32 literals
    s = re.sub(r"(?<![\w.])(\d+)i32\b", r"\1", s)                       # Int32 literals
    # implicit products: a numeric literal (possibly with exponent) followed by a name or '('
    s = re.sub(_NUM + r"((?:[eE][-+]?\d+)?)(?=[A-Za-z_Ͱ-Ͽᴀ-ᶿ(])",
               lambda m: m.group(1) + m.group(2) + ("*" if not (m.group(2) == "" and
                                                              re.match(r"[eE]", s[m.end():m.end() + 1] or "x"))
                                                    else ""), s)
    s = s.replace("^", "**")
    s = _literal_powers(s)
    s = s.replace("&&", " and ").replace("||", " or ")
    s = re.sub(r"!(?!=)", " not ", s)
    s = s.replace("÷", "//")
    s = re.sub(r"\btrue\b", "True", s)
    s = re.sub(r"\bfalse\b", "False", s)
    s = re.sub(r"\bnothing\b", "None", s)
    s = re.sub(r"\bFloat32\(", "_f32(", s)
    s = re.sub(r"\bFloat64\(", "_f64(", s)
    s = _ternary(s)
    # characters Julia allows in names and Python does not (e.g. the ∂ of ∂ξ∂x)
    s = "".join(c if ord(c) < 128 or ("a" + c).isidentifier() else f"_u{ord(c):04x}_" for c in s)
    return s


def _strip_macros(s: str) -> str:
    s = re.sub(r"@(inbounds|fastmath|inline|view)\s+", "", s).strip()  # a view reads what the slice does
    # a kernel launch of a host function: @cuda <keyword = value ...> f(args) -> _cuda(f, args)
    m = re.match(r"@cuda\s+(.*)$", s)
    if m:
        rest = m.group(1)
        while True:
            k = re.match(r"\w+\s*=\s*[\w.()]+\s+(?=\w)", rest)
            if not k:
                break
            rest = rest[k.end():]
        c = re.match(r"(\w+)\((.*)\)\s*$", rest)
        if not c:
            raise ValueError(f"unrecognised launch: {s}")
        s = f"_cuda({c.group(1)}, {c.group(2)})"
    return s


def _strip_annot(lhs: str) -> str:
    return re.sub(r"::\s*\w+(\{[^}]*\})?", "", lhs).strip()


_expr = expr  # for translate_script, whose local name expr selects the typed form


def _top_colon(s: str) -> int:
    """Index of the first ':' outside brackets, or -1."""
    d = 0
    for i, ch in enumerate(s):
        if ch in _OPEN:
            d += 1
        elif ch in _CLOSE:
            d -= 1
        elif ch == ":" and d == 0:
            return i
    return -1


def _loops(spec: str, ex) -> list[tuple[str, str]]:
    """`k in K_in, j = 1:n, i ∈ a:b` -> [(var, Python iterable), ...], the first outermost:
    a:b is range(a, b + 1), anything else (a range variable) is iterated as it is."""
    out = []
    for part in (t.strip() for t in re.split(r",(?![^()\[\]]*[)\]])", spec)):
        v, rng = re.split(r"\s*(?:∈|=|\bin\b)\s*", part, maxsplit=1)
        c = _top_colon(rng)
        out.append((v, f"range({ex(rng[:c].strip())}, ({ex(rng[c + 1:].strip())}) + 1)" if c >= 0 else ex(rng)))
    return out

_ANNOT = re.compile(r"^\s*([^\W\d]\w*)\s*::\s*Float(32|64)\s*$")


def translate(src: str, typed: bool = False) -> str:
    """Python source of every function of a Julia kernel file (top-level code is skipped).
    typed: Julia's element types kept (literals, `x::Float32` locals converting on every
    assignment, temporaries) for an evaluation in Float32 / Float64 NumPy scalars."""
    expr_ = (lambda e: expr(e, True)) if typed else expr
    out: list[str] = []
    stack: list[str] = []
    types: dict[str, str] = {}  # the declared Float32 / Float64 locals of the current function
    # indentation levels opened by each block: begin .. end none, a loop over n variables n
    levels = lambda k: 0 if k == "begin" else (int(k[4:]) if k.startswith("for:") else 1)
    pad = lambda: "    " * sum(levels(k) for k in stack)
    last_expr = None  # index in out of the function body's last statement if it is a bare expression
    for raw in logical_lines(src):
        s = _strip_macros(raw)
        if stack and s != "end":
            last_expr = None
        if not stack:
            m = re.match(r"function\s+(\w+)\s*\((.*)\)\s*$", s)
            if m:
                out.append(f"def {m.group(1)}({_strip_annot(m.group(2))}):")
                stack.append("function")
                types = {}
            continue
        if s == "end":
            stack.pop()
            if not stack:
                # Julia returns the value of a function's last expression
                if last_expr is not None:
                    out[last_expr] = "    return " + out[last_expr].strip()
                out.append("")
            last_expr = None
            continue
        if re.match(r"function\b", s):
            raise ValueError(f"nested function: {s}")
        if s == "begin":
            stack.append("begin")
            continue
        m = re.match(r"if\s+(.*)$", s)
        if m:
            out.append(pad() + f"if {expr_(m.group(1))}:")
            stack.append("if")
            continue
        m = re.match(r"elseif\s+(.*)$", s)
        if m:
            out.append(pad()[4:] + f"elif {expr_(m.group(1))}:")
            continue
        if s == "else":
            out.append(pad()[4:] + "else:")
            continue
        m = re.match(r"for\s+(.*)$", s)
        if m:
            base = pad()
            loops = _loops(m.group(1), expr_)
            for k, (v, it) in enumerate(loops):
                out.append(base + "    " * k + f"for {v} in {it}:")
            stack.append(f"for:{len(loops)}")
            continue
        if s == "return" or s.startswith("return "):
            rest = s[len("return"):].strip()
            out.append(pad() + ("return" if not rest else f"return {expr_(rest)}"))
            continue
        m = re.match(r"(.+?)\s*\.=\s*(.+)$", s)
        if m:
            out.append(pad() + f"{expr_(m.group(1))}._fill({expr_(m.group(2))})")
            continue
        m = re.match(r"(.+?)\s*(\+=|-=|\*=|/=)\s*(.+)$", s)
        if m:
            lhs = expr_(_strip_annot(m.group(1)))
            if typed and lhs in types:  # x op= e assigns x op e converted to x's declared type
                out.append(pad() + f"{lhs} = _f{types[lhs]}({lhs} {m.group(2)[0]} ({expr_(m.group(3))}))")
            else:
                out.append(pad() + f"{lhs} {m.group(2)} {expr_(m.group(3))}")
            continue
        m = re.match(r"([^=<>!]+?)\s*=(?!=)\s*(.+)$", s)
        if m:
            a = _ANNOT.match(m.group(1))
            lhs = expr_(_strip_annot(m.group(1)))
            if typed and a:
                types[lhs] = a.group(2)
            rhs, c = m.group(2), _top_colon(m.group(2))
            if c >= 0 and "?" not in rhs:  # a range a:b
                out.append(pad() + f"{lhs} = range({expr_(rhs[:c].strip())}, ({expr_(rhs[c + 1:].strip())}) + 1)")
            elif typed and lhs in types:
                out.append(pad() + f"{lhs} = _f{types[lhs]}({expr_(rhs)})")
            else:
                out.append(pad() + f"{lhs} = {expr_(rhs)}")
            continue
        out.append(pad() + expr_(s))
        if len(stack) == 1:
            last_expr = len(out) - 1
    if stack:
        raise ValueError(f"unterminated blocks: {stack}")
    # a function whose body is empty after translation still needs a statement
    fixed = []
    for i, l in enumerate(out):
        fixed.append(l)
        if l.rstrip().endswith(":") and (i + 1 == len(out) or len(out[i + 1]) - len(out[i + 1].lstrip()) <=
                                          len(l) - len(l.lstrip())):
            fixed.append(" " * (len(l) - len(l.lstrip()) + 4) + "pass")
    return "\n".join(fixed) + "\n"


def translate_script(src: str, first: int, last: int, typed: bool = False) -> str:
    """Python of the top-level statements of lines first..last (1-based) of a Julia script:
    function definitions, assignments, `@.` broadcasts (-> _bset(lhs, rhs), elementwise on whole
    arrays, the same operations per element), loops `for k ∈ a:b, j ∈ c:d, ...` (nested, the
    first variable outermost) and ifs. typed: Julia's element types kept, as translate()."""
    expr = (lambda e: _expr(e, True)) if typed else _expr
    lines = src.splitlines()[first - 1:last]
    out: list[str] = []
    stack: list[int] = []  # indentation levels opened by each block
    depth = lambda: sum(stack)
    last_expr = None
    in_fun = []
    for raw in logical_lines("\n".join(lines)):
        s = _strip_macros(raw)
        if s != "end":
            last_expr = None
        if s == "end":
            n = stack.pop()
            if in_fun and len(stack) == in_fun[-1]:
                if last_expr is not None:
                    out[last_expr] = "    " * (depth() + 1) + "return " + out[last_expr].strip()
                in_fun.pop()
            last_expr = None
            continue
        pad = "    " * depth()
        m = re.match(r"function\s+(\w+)\s*\((.*)\)\s*$", s)
        if m:
            out.append(pad + f"def {m.group(1)}({_strip_annot(m.group(2))}):")
            in_fun.append(len(stack))
            stack.append(1)
            continue
        m = re.match(r"for\s+(.*)$", s)
        if m:
            specs = [t.strip() for t in re.split(r",(?![^()\[\]]*[)\]])", m.group(1))]
            for k, spec in enumerate(specs):
                v, rng = re.split(r"\s*(?:∈|=|\bin\b)\s*", spec, maxsplit=1)
                a, b = rng.split(":", 1)
                out.append("    " * (depth() + k) + f"for {v} in range({expr(a)}, ({expr(b)}) + 1):")
            stack.append(len(specs))
            continue
        m = re.match(r"if\s+(.*)$", s)
        if m:
            out.append(pad + f"if {expr(m.group(1))}:")
            stack.append(1)
            continue
        if s.startswith("return"):
            rest = s[len("return"):].strip()
            out.append(pad + ("return" if not rest else f"return {expr(rest)}"))
            continue
        m = re.match(r"@\.\s*(.+?)\s*=(?!=)\s*(.+)$", s)
        if m:
            out.append(pad + f"_bset({expr(m.group(1))}, {expr(m.group(2))})")
            continue
        m = re.match(r"(\w+)\s*\.([-+*/])=\s*(.+)$", s)  # x ./= e: elementwise x = x / e
        if m:
            out.append(pad + f"_bset({m.group(1)}, {m.group(1)} {m.group(2)} ({expr(m.group(3))}))")
            continue
        m = re.match(r"([^=<>!]+?)\s*=(?!=)\s*(.+)$", s)
        if m:
            out.append(pad + f"{expr(_strip_annot(m.group(1)))} = {expr(m.group(2))}")
            continue
        out.append(pad + expr(s))
        if in_fun and len(stack) == in_fun[-1] + 1:
            last_expr = len(out) - 1
    if stack:
        raise ValueError(f"unterminated blocks: {stack}")
    return "\n".join(out) + "\n"


# the metric and Jacobian computation of parse_mesh.jl (its CD6 / CD2 stencils of the
# coordinates, J and the J^-1-scaled metrics), without the file output that follows
METRIC_LINES = (139, 248)
# the same computation in SCU-benchmark/readfort.jl (Float32 coefficients): its CD6 / CD2
# functions and the body of computeMetrics before its file output
READFORT = "SCU-benchmark/readfort.jl"
READFORT_LINES = ((104, 117), (120, 208))
# the ghost coordinates: readfort.jl's generateXYZ after reading the file (point reflection,
# edge completion, then ./= 1000) and solver.jl's extrapolation of the coordinates it reads
READFORT_GHOST_LINES = (34, 99)
# parse_mesh.jl's flat-plate coordinates: stretching_y, the mapping of every cell, then the
# ghost reflections (its constants Lx, Ly, Lz, stretch_factor_y become parameters)
FLAT_PLATE_LINES = ((38, 41), (46, 136))
EXTRAPOLATION = ("solver.jl", "function extrapolation(")


def _function_text(src: str, head: str) -> str:
    """The top-level function starting with `head`, through its closing `end` line."""
    i = src.index(head)
    j = src.index("\nend", i)
    return src[i:j + 4] + "\n"


def translate_tree(root: Path, corrected: bool = False, typed: bool = False) -> str:
    parts = ["# Generated by oracle/ref_jl/jl2py.py from the reference's Julia kernels; do not edit.\n"]
    if corrected:
        parts.append("# With CORRECTIONS applied (FVM.jl).\n")
    if typed:
        parts.append("# Typed: Julia's Float32 / Float64 literals, locals and temporaries kept.\n")
    for name in FILES:
        src = (root / name).read_text()
        parts.append(f"# ---- {name}\n")
        parts.append(translate(apply_corrections(name, src) if corrected else src, typed))
    a, b = METRIC_LINES
    parts.append(f"# ---- parse_mesh.jl:{a}-{b}, as the body of _metrics()\n")
    body = translate_script((root / "parse_mesh.jl").read_text(), a, b, typed)
    parts.append("def _metrics(x, y, z):\n" + "".join("    " + l + "\n" if l else "\n" for l in body.splitlines()) +
                 "    return (dξdx, dξdy, dξdz, dηdx, dηdy, dηdz, dζdx, dζdy, dζdz), J\n")
    rf = (root / READFORT).read_text()
    parts.append(f"# ---- {READFORT}:" + ", ".join(f"{a}-{b}" for a, b in READFORT_LINES) +
                 ", as the body of _metrics_readfort()\n")
    body = "".join(translate_script(rf, a, b, typed) for a, b in READFORT_LINES)
    parts.append("def _metrics_readfort(x, y, z):\n" + "".join("    " + l + "\n" if l else "\n" for l in body.splitlines()) +
                 "    return (dξdx, dξdy, dξdz, dηdx, dηdy, dηdz, dζdx, dζdy, dζdz), J\n")
    a, b = READFORT_GHOST_LINES
    parts.append(f"# ---- {READFORT}:{a}-{b}, as the body of _ghosts_readfort()\n")
    body = translate_script(rf, a, b, typed)
    parts.append("def _ghosts_readfort(x, y, z):\n" + "".join("    " + l + "\n" if l else "\n" for l in body.splitlines()) +
                 "    return x, y, z\n")
    pm = (root / "parse_mesh.jl").read_text()
    parts.append("# ---- parse_mesh.jl:" + ", ".join(f"{a}-{b}" for a, b in FLAT_PLATE_LINES) +
                 ", as the body of _flat_plate()\n")
    body = "".join(translate_script(pm, a, b, typed) for a, b in FLAT_PLATE_LINES)
    parts.append("def _flat_plate(x, y, z, Lx, Ly, Lz, stretch_factor_y):\n" +
                 "".join("    " + l + "\n" if l else "\n" for l in body.splitlines()) + "    return x, y, z\n")
    f, head = EXTRAPOLATION
    parts.append(f"# ---- {f}: {head.rstrip('(')}\n")
    parts.append(translate(_function_text((root / f).read_text(), head), typed))
    return "\n".join(parts)


def main(argv=None) -> None:
    argv = sys.argv[1:] if argv is None else argv
    corrected, typed = "--corrected" in argv, "--typed" in argv
    argv = [a for a in argv if a not in ("--corrected", "--typed")]
    root = Path(argv[0])
    out = Path(argv[1]) if len(argv) > 1 else Path(__file__).resolve().parent.parent / "_ref" / "jl_kernels.py"
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(translate_tree(root, corrected, typed))
    print(out)


if __name__ == "__main__":
    main()

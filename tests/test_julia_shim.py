"""The Julia ccall shim (fluxoptics.jl_gb300/julia/FluxOpticsGB300.jl) against the
C ABI it binds (include/fluxoptics_gb300.h).  Julia is not installed here, so the
shim is checked as text: every `ccall((:fo_..., LIB), R, (T1, T2, ...), ...)`
must name a declared entry point, with the declared number of arguments, a
matching return type and argument types of the right kind (Cint for int, Cdouble
for double, a Ptr/Ref for every pointer or opaque handle)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fluxoptics_gb300.h")
SHIM = os.path.join(ROOT, "fluxoptics.jl_gb300", "julia", "FluxOpticsGB300.jl")


def _strip_c_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def header_decls():
    """name -> (return type, [argument types])."""
    src = _strip_c_comments(open(HEADER).read())
    handles = set(re.findall(r"typedef\s+struct\s+\w+\s*\*\s*(\w+)\s*;", src))
    decls = {}
    for ret, name, args in re.findall(r"FO_API\s+([\w\s\*]+?)\s*\b(fo_\w+)\s*\(([^)]*)\)\s*;", src):
        args = " ".join(args.split())
        types = []
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                m = re.match(r"(.*?)(\w+)$", a)  # drop the parameter name
                types.append(" ".join(m.group(1).split()) if m and m.group(1).strip() else a)
        decls[name] = (" ".join(ret.split()), types)
    return decls, handles


def _balanced(s, i):
    """Index one past the parenthesis group starting at s[i] == '('."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced parentheses")


def _split_top(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def shim_ccalls():
    """[(symbol, return type, [argument types], line)] of every ccall in the shim."""
    src = open(SHIM).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(fo_\w+),\s*LIB\),\s*", src):
        i = m.end()
        j = src.index(",", i)
        ret = src[i:j].strip()
        k = j + 1
        while src[k].isspace():
            k += 1
        assert src[k] == "(", f"argument-type tuple of {m.group(1)} not found"
        end = _balanced(src, k)
        calls.append((m.group(1), ret, _split_top(src[k + 1:end - 1]), src.count("\n", 0, m.start()) + 1))
    return calls


def _compatible(ctype, jtype, handles):
    base = ctype.replace("const ", "").strip()
    if "*" in base or base in handles:
        return jtype.startswith("Ptr{") or jtype.startswith("Ref{")
    return {"int": "Cint", "double": "Cdouble", "long long": "Clonglong", "size_t": "Csize_t",
            "float": "Cfloat"}.get(base) == jtype


def test_shim_binds_declared_entry_points():
    decls, handles = header_decls()
    calls = shim_ccalls()
    assert len(calls) > 40
    for sym, ret, args, line in calls:
        assert sym in decls, f"line {line}: {sym} is not declared in the header"
        cret, cargs = decls[sym]
        assert len(args) == len(cargs), f"line {line}: {sym} takes {len(cargs)} arguments, the shim passes {len(args)}"
        want_ret = "Cstring" if cret == "const char*" else "Cint"
        assert ret == want_ret, f"line {line}: {sym} returns {cret}, the shim expects {ret}"
        for n, (ct, jt) in enumerate(zip(cargs, args)):
            assert _compatible(ct, jt, handles), f"line {line}: {sym} argument {n + 1} is {ct!r}, shim has {jt!r}"


@pytest.mark.parametrize("sym", [
    "fo_bpm_create", "fo_bpm_forward", "fo_bpm_backward", "fo_bpm_destroy",
    "fo_sid_create", "fo_sid_forward", "fo_sid_backward", "fo_sid_destroy",
    "fo_chain_forward_sid", "fo_chain_backward_ex", "fo_chain_withgradient_sid", "fo_chain_withgradient_sfd",
    "fo_fista_step", "fo_fista_clamp_step", "fo_clamp", "fo_tv_create_ex", "fo_tv_apply", "fo_tv_destroy",
])
def test_shim_covers_the_hot_path(sym):
    assert sym in {c[0] for c in shim_ccalls()}, f"{sym} has no Julia binding"


def test_header_parser_sees_every_entry_point():
    decls, _ = header_decls()
    src = _strip_c_comments(open(HEADER).read())
    uses = [ln for ln in src.splitlines() if "FO_API" in ln and not ln.lstrip().startswith("#")]
    assert len(decls) == len(uses)
    assert decls["fo_fista_step"][1] == ["float*", "float*", "float*", "const float*", "long long", "double",
                                         "double*", "void*"]

"""Static checks of the Julia ccall shim (Julia is not installed here, so the
shim cannot run): its C struct mirrors have the header's fields in the header's
order with matching types, every symbol it ccalls is declared by the header, and
every ccall's return type and argument types agree with the C prototype."""
import re
from pathlib import Path

import cheader

ROOT = Path(__file__).resolve().parent.parent
HEADER = (ROOT / "include" / "helmgpu.h").read_text()
SHIM = (ROOT / "helmholtz.jl_gb300" / "julia" / "HelmholtzGB300.jl").read_text()

C2J = {"int32_t": "Int32", "int64_t": "Int64", "double": "Float64", "const double*": "Ptr{Float64}"}


def c_fields(name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), HEADER, re.S).group(1)
    out = []
    for line in body.splitlines():
        line = re.sub(r"/\*.*?\*/", "", line).strip()
        if not line:
            continue
        m = re.match(r"(const double\*|int32_t|int64_t|double)\s+(\w+)(\[(\d+)\])?;", line)
        assert m, line
        ty = C2J[m.group(1)]
        if m.group(4):
            ty = "NTuple{%s,%s}" % (m.group(4), ty)
        out.append((m.group(2), ty))
    return out


def jl_fields(name):
    body = re.search(r"(?:mutable )?struct %s\n(.*?)\nend" % name, SHIM, re.S).group(1)
    out = []
    for line in body.splitlines():
        line = line.split("#")[0].strip()
        if line:
            n, t = line.split("::")
            out.append((n.strip(), t.strip()))
    return out


def test_struct_mirrors_match_header():
    for c, j in (("hz_problem", "HzProblem"), ("hz_options", "HzOptions"), ("hz_stats", "HzStats")):
        assert c_fields(c) == jl_fields(j), (c, c_fields(c), jl_fields(j))


def test_ccalled_symbols_are_declared():
    called = set(re.findall(r"ccall\(\(:(\w+),", SHIM))
    declared = set(re.findall(r"\b(hz_\w+)\(", HEADER))
    assert called, "no ccall found"
    assert called <= declared, called - declared


def test_option_constants_match_header():
    for name, val in re.findall(r"const (HZ_\w+) = Int32\((-?\d+)\)", SHIM):
        m = re.search(r"#define %s \(?(-?\d+)\)?" % name, HEADER)
        assert m and int(m.group(1)) == int(val), name


# C parameter / return types and the Julia ccall types that pass them correctly
# (complex arrays travel as interleaved double pairs: Ptr{ComplexF64} for double*).
C2CCALL = {
    "void": {"Cvoid"},
    "int": {"Cint", "Int32"},
    "int32_t": {"Int32", "Cint"},
    "int64_t": {"Int64"},
    "double": {"Float64", "Cdouble"},
    "const char*": {"Cstring", "Ptr{UInt8}"},
    "char*": {"Ptr{UInt8}"},
    "double*": {"Ptr{Float64}", "Ptr{ComplexF64}", "Ref{Float64}"},
    "const double*": {"Ptr{Float64}", "Ptr{ComplexF64}"},
    "float*": {"Ptr{Float32}"},
    "const float*": {"Ptr{Float32}"},
    "int32_t*": {"Ptr{Int32}", "Ref{Int32}"},
    "int64_t*": {"Ptr{Int64}", "Ref{Int64}"},
    "const int64_t*": {"Ptr{Int64}"},
    "void*": {"Ptr{Cvoid}"},
    "hz_handle*": {"Ptr{Cvoid}"},
    "const hz_handle*": {"Ptr{Cvoid}"},
    "hz_net*": {"Ptr{Cvoid}"},
    "const hz_net*": {"Ptr{Cvoid}"},
    "hz_handle**": {"Ref{Ptr{Cvoid}}"},
    "hz_net**": {"Ref{Ptr{Cvoid}}"},
    "const hz_problem*": {"Ref{HzProblem}"},
    "hz_options*": {"Ref{HzOptions}"},
    "const hz_options*": {"Ref{HzOptions}"},
    "hz_stats*": {"Ref{HzStats}"},
}


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        depth += ch in "({["
        depth -= ch in ")}]"
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    return parts + ([cur.strip()] if cur.strip() else [])


def _ccalls():
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*libhelmgpu\),", SHIM):
        i, depth = m.end(), 0
        for k in range(i, len(SHIM)):
            depth += SHIM[k] in "({["
            depth -= SHIM[k] in ")}]"
            if SHIM[k] == "," and depth == 0:
                break
        ret = SHIM[i:k].strip()
        j = k + 1
        while SHIM[j].isspace():
            j += 1
        assert SHIM[j] == "(", m.group(1)
        depth = 0
        for e in range(j, len(SHIM)):
            depth += SHIM[e] in "({["
            depth -= SHIM[e] in ")}]"
            if depth == 0:
                break
        calls.append((m.group(1), ret, _split_top(SHIM[j + 1:e])))
    return calls


def test_ccall_signatures_match_prototypes():
    """Every ccall passes as many arguments as the C prototype takes, each with a
    Julia type that has the C type's size and meaning, and reads the right return type."""
    protos = cheader.prototypes()
    calls = _ccalls()
    assert len(calls) >= 20
    for name, ret, args in calls:
        cret, cargs = protos[name]
        assert ret in C2CCALL[cret], (name, ret, cret)
        assert len(args) == len(cargs), (name, args, cargs)
        for a, c in zip(args, cargs):
            assert a in C2CCALL[c], (name, a, c)

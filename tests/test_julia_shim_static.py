"""Static checks of the Julia ccall shim (Julia is not installed here, so the
shim cannot run): its C struct mirrors have the header's fields in the header's
order with matching types, and every symbol it ccalls is declared by the header."""
import re
from pathlib import Path

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

"""The Julia shim's C calls against the C ABI, checked statically.

julia/FlexShellGPU.jl binds the reference's Julia API to the C ABI of
include/flexshell.h through ccall.  No Julia toolchain is available to run
it, and a wrong ccall does not fail loudly: a wrong argument count, type or
width, a struct mirror whose fields drift from the C struct, or a constant
that differs from the header's corrupts the call silently.  These tests
parse every ccall of the shim and check it against the header's prototype:

* the symbol is declared in the header (whose exports the ABI test checks
  against the built library);
* the return type is int and the argument tuple has the prototype's arity;
* each argument type matches the C parameter (width and signedness of
  scalars, pointer depth and pointee of pointers; Ptr{Cvoid} is an address
  and stands for any pointer);
* the three struct mirrors (FsShellParams, FsLayupGroup, FsBeamSection) have
  the C structs' fields in order, with the same names, types and array
  lengths, and the ctypes mirror the GPU tests use has the same size;
* every FS_ constant the shim defines has the header's value.
"""
import ctypes
import os
import re

import pytest

from flexshell import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "flexshell.h")
SHIM = os.path.join(ROOT, "finetoolsflexstructures.jl_gb300", "julia", "FlexShellGPU.jl")


def _c_source():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def _c_param(p):
    """'const double *const *xyz' -> ('double', 2)."""
    depth = p.count("*")
    words = [w for w in re.split(r"[\s*]+", p) if w and w != "const"]
    if len(words) == 1 and words[0] == "void" and depth == 0:
        return None
    return words[0], depth


def _prototypes():
    protos = {}
    for m in re.finditer(r"\b(\w+)\s+(fs_\w+)\s*\(([^;{)]*)\)\s*;", _c_source()):
        ret, name, params = m.groups()
        ps = [_c_param(p) for p in params.split(",") if p.strip()]
        protos[name] = (ret, [p for p in ps if p is not None])
    return protos


def _split_top(s):
    """Split at commas outside (), {} and []."""
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


def _ccalls():
    """(symbol, return type, [argument types], number of arguments, line)."""
    src = open(SHIM).read()
    calls = []
    for m in re.finditer(r"\bccall\(", src):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        parts = _split_top(src[m.end():i - 1])
        sym = re.match(r"\(\s*:(\w+)\s*,\s*libflexshell\s*\)", parts[0])
        assert sym, parts[0]
        tup = parts[2].strip()
        assert tup.startswith("(") and tup.endswith(")"), tup
        types = _split_top(tup[1:-1])
        calls.append((sym.group(1), parts[1], types, len(parts) - 3, src.count("\n", 0, m.start()) + 1))
    return calls


SCALARS = {
    "Cint": {"int", "int32_t"}, "Int32": {"int", "int32_t"}, "Int64": {"int64_t"}, "UInt64": {"uint64_t"},
    "Float64": {"double"}, "Cdouble": {"double"}, "Csize_t": {"size_t"}, "UInt8": {"uint8_t", "char"},
    "Cchar": {"char"}, "FsShellParams": {"fs_shell_params"}, "FsLayupGroup": {"fs_layup_group"},
    "FsBeamSection": {"fs_beam_section"},
}


def _matches(jt, c):
    base, depth = c
    m = re.fullmatch(r"(Ptr|Ref)\{(.*)\}", jt)
    if m:
        inner = m.group(2)
        if depth < 1:
            return False
        if inner == "Cvoid":
            return True
        return _matches(inner, (base, depth - 1))
    return depth == 0 and base in SCALARS.get(jt, ())


def test_every_ccall_matches_its_prototype():
    protos = _prototypes()
    calls = _ccalls()
    assert len(calls) >= 25
    for sym, ret, types, nargs, line in calls:
        assert sym in protos, "line %d: %s is not declared in flexshell.h" % (line, sym)
        cret, cparams = protos[sym]
        assert cret == "int" and ret == "Cint", (line, sym, ret)
        assert len(types) == len(cparams), "line %d: %s takes %d arguments, the shim passes %d types" % (
            line, sym, len(cparams), len(types))
        assert nargs == len(types), "line %d: %s: %d types, %d arguments" % (line, sym, len(types), nargs)
        for k, (jt, c) in enumerate(zip(types, cparams)):
            assert _matches(jt, c), "line %d: %s argument %d: Julia %s against C %s%s" % (
                line, sym, k + 1, jt, c[0], " *" * c[1])


def test_shim_binds_the_reference_facing_entry_points():
    # the stiffness, mass, restoring force, explicit loop, eigen and
    # resultant entry points of the shells and the beam are all bound
    protos = _prototypes()
    called = {c[0] for c in _ccalls()}
    for sym in ("fs_ctx_create", "fs_ctx_destroy", "fs_mesh_set", "fs_params_set", "fs_layups_set",
                "fs_normals_set", "fs_stiffness", "fs_mass", "fs_matrix_copy", "fs_restoring_force",
                "fs_explicit_setup", "fs_explicit_run", "fs_shift_factor", "fs_shift_solve",
                "fs_resultants", "fs_beam_setup", "fs_beam_matrix", "fs_beam_restoringforce"):
        assert sym in called and sym in protos, sym


def _c_struct(name):
    m = re.search(r"typedef\s+struct\s*\{([^{}]*)\}\s*" + name + r"\s*;", _c_source())
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, rest = decl.split(None, 1)
        for f in rest.split(","):
            fm = re.fullmatch(r"\s*(\w+)\s*(?:\[(\d+)\])?\s*", f)
            assert fm, f
            fields.append((fm.group(1), ctype, int(fm.group(2) or 1)))
    return fields


def _julia_struct(name):
    m = re.search(r"^struct " + name + r"\n(.*?)^end", open(SHIM).read(), flags=re.S | re.M)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("#")[0].strip()
        if not line:
            continue
        fm = re.fullmatch(r"(\w+)::(Int32|Float64|NTuple\{(\d+),\s*(Int32|Float64)\})", line)
        assert fm, line
        jt = fm.group(4) or fm.group(2)
        fields.append((fm.group(1), {"Int32": "int32_t", "Float64": "double"}[jt], int(fm.group(3) or 1)))
    return fields


@pytest.mark.parametrize("jname,cname", [("FsShellParams", "fs_shell_params"),
                                         ("FsLayupGroup", "fs_layup_group"),
                                         ("FsBeamSection", "fs_beam_section")])
def test_struct_mirrors_match_the_c_structs(jname, cname):
    c = _c_struct(cname)
    assert _julia_struct(jname) == c
    # the ctypes mirror (used by the GPU tests) has the C layout's size:
    # int32 and double fields, 8-byte aligned
    size = 0
    for _, t, n in c:
        w = 4 if t == "int32_t" else 8
        size = (size + w - 1) // w * w + w * n
    size = (size + 7) // 8 * 8
    assert ctypes.sizeof(getattr(_abi, cname)) == size


def test_julia_constants_have_the_header_values():
    c = {k: int(v) for k, v in re.findall(r"#define\s+(FS_\w+)\s+(-?\d+)\b", open(HEADER).read())}
    src = open(SHIM).read()
    seen = 0
    for names, values in re.findall(r"^const\s+(FS_[\w, ]+?)\s*=\s*([-\d, ]+)$", src, flags=re.M):
        ns = [n.strip() for n in names.split(",")]
        vs = [int(v) for v in values.split(",")]
        assert len(ns) == len(vs), names
        for n, v in zip(ns, vs):
            assert n in c and c[n] == v, (n, v, c.get(n))
            seen += 1
    assert seen >= 17

"""CPU checks of the C-ABI library: it builds, loads, and exports every
function that include/flexshell.h declares (no compute call: no GPU here)."""
import ctypes
import os
import re

import numpy as np

from flexshell import _abi, _lib, femm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "flexshell.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^int\s+(fs_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 20
    L = _lib.lib()
    for n in names:
        assert hasattr(L, n), n


def test_struct_layouts_match_header():
    # fs_shell_params: 2 int32 + 3 doubles + 9 + 4 + 2 doubles
    assert ctypes.sizeof(_abi.fs_shell_params) == 8 + 8 * (3 + 9 + 4 + 2)
    assert ctypes.sizeof(_abi.fs_layup_group) == 8 * (9 * 3 + 4 + 9 + 3)
    assert ctypes.sizeof(_abi.fs_beam_section) == 8 * 10


def test_stab_fun_family():
    assert abs(femm.stab_coefficient(lambda t, h: t ** 2 / (t ** 2 + 0.2 * h ** 2), 0.1) - 0.2) < 1e-14
    assert femm.stab_coefficient(None, 0.1) == 0.1
    try:
        femm.stab_coefficient(lambda t, h: t / (t + h), 0.1)
    except ValueError:
        pass
    else:
        raise AssertionError("closure outside the family accepted")


def test_numberdofs_matches_finetools_rule():
    fx = np.zeros((3, 6), bool)
    fx[1, [0, 2]] = True
    from flexshell import mesh
    d, nf = mesh.numberdofs(fx)
    assert nf == 16
    assert d[0].tolist() == [1, 2, 3, 4, 5, 6]
    assert d[1].tolist() == [17, 7, 18, 8, 9, 10]
    assert d[2].tolist() == [11, 12, 13, 14, 15, 16]


def _ctypes_matches(expr, c):
    """A ctypes argtype expression of flexshell/_lib.py against a C parameter
    (base type, pointer depth); c_void_p is an address, so it stands for any
    pointer."""
    base, depth = c
    scalars = {"ctypes.c_int": {"int", "int32_t"}, "ctypes.c_int32": {"int", "int32_t"},
               "ctypes.c_int64": {"int64_t"}, "ctypes.c_uint64": {"uint64_t"}, "ctypes.c_double": {"double"},
               "ctypes.c_size_t": {"size_t"}}
    if expr in ("vp", "ctypes.c_void_p"):
        return depth >= 1
    if expr == "ctypes.c_char_p":
        return depth == 1 and base == "char"
    if expr == "_c_i64_p":
        return depth == 1 and base == "int64_t"
    m = re.fullmatch(r"ctypes\.POINTER\((.*)\)", expr)
    if m:
        inner = m.group(1)
        if inner.startswith("_abi."):
            return depth == 1 and base == inner[5:]
        return depth >= 1 and _ctypes_matches(inner, (base, depth - 1))
    return depth == 0 and base in scalars.get(expr, ())


def test_ctypes_argtypes_match_the_prototypes():
    # every declared function has argtypes in the Python mirror (ctypes'
    # default int conversion would truncate 64-bit arguments), with the
    # prototype's arity and, argument by argument, its width or pointer depth
    from test_julia_shim import _prototypes, _split_top
    protos = _prototypes()
    src = open(os.path.join(ROOT, "finetoolsflexstructures.jl_gb300", "flexshell", "_lib.py")).read()
    decl = {m.group(1): _split_top(m.group(2))
            for m in re.finditer(r"L\.(fs_\w+)\.argtypes\s*=\s*\[(.*?)\]\n", src, flags=re.S)}
    assert set(decl) == set(protos), sorted(set(decl) ^ set(protos))
    for name, types in decl.items():
        cparams = protos[name][1]
        assert len(types) == len(cparams), (name, len(types), len(cparams))
        for k, (t, c) in enumerate(zip(types, cparams)):
            assert _ctypes_matches(t, c), "%s argument %d: ctypes %s against C %s%s" % (
                name, k + 1, t, c[0], " *" * c[1])


def test_without_a_gpu_the_library_fails_loudly():
    # the library has no CPU path: without a CUDA device no context can be
    # created, so a FEMM cannot be made and nothing is computed elsewhere
    # (skipped where a device is present)
    from flexshell._lib import Context, FlexShellError
    try:
        ctx = Context(0)
    except FlexShellError as e:
        err = e
    else:
        ctx.close()
        import pytest
        pytest.skip("a CUDA device is present")
    assert "cannot create a context" in str(err)
    import pytest
    from flexshell import materials
    with pytest.raises(FlexShellError):
        femm.FEMMShellT3FF(np.array([[1, 2, 3]]), 0.01, materials.MatDeforElastIso(2e11, 0.3, 7850.0))


def test_input_cache_sees_in_place_changes_and_replacements():
    # the mirror re-uploads geom0 / dchi exactly when their content differs
    # from what it uploaded last: an in-place move, an in-place renumbering
    # (which keeps the dof numbers' sum) and a new shape are seen; an equal
    # copy is not an upload
    from flexshell._lib import InputCache
    c = InputCache()
    a = np.asfortranarray(np.arange(12.0).reshape(4, 3))
    assert c.stale(a)
    c.store(a)
    assert not c.stale(a)
    a[2, 1] += 1e-9
    assert c.stale(a)
    c.store(a)
    assert not c.stale(a.copy())
    d = np.asfortranarray(np.arange(1, 13, dtype=np.int64).reshape(4, 3))
    c.store(d)
    d[[0, 1]] = d[[1, 0]]
    assert c.stale(d) and c.copy.sum() == d.sum()
    assert c.stale(np.zeros((5, 3)))
    c.clear()
    assert c.stale(d)

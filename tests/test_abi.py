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

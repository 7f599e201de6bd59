"""The allocation-free stiffness entry point (fs_stiffness_values_noalloc).

It serves callers that cannot let the library allocate device memory when
they ask for a stiffness (their own pool allocator owns the GPU memory, or
their solver loop runs under a fixed memory budget).  The test calls it
through the C ABI, twice in a row, into a device buffer the caller owns, and
checks the values against the regular fs_stiffness entry point bit for bit
(both run the same element and gather kernels); a beam context and a mesh
beyond the fixed array are rejected before any launch.  This file is
collected last so that a run stopping at the first failure has run every
other test before it.
"""
import ctypes

import numpy as np
import pytest

import flexshell as F
from flexshell import _abi, materials
from flexshell._lib import FlexShellError, ptr
import problems as PB

pytestmark = pytest.mark.gpu

TOL = {_abi.FS_FP64: 1e-12, _abi.FS_MIXED: 1e-6, _abi.FS_MIXED_COMP: 1e-6}


def _femm(n, quads):
    xyz, conn, dof, nfree = PB.jittered_plate(n, quads, wavy=0.01, seed=11)
    mat = materials.MatDeforElastIso(200e9, 0.3, 7850.0)
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(conn, 0.005, mat)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    return femm, geom0, dchi


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("precision", [_abi.FS_FP64, _abi.FS_MIXED, _abi.FS_MIXED_COMP])
def test_noalloc_matches_regular_entry_point(quads, precision):
    import torch
    femm, geom0, dchi = _femm(16, quads)
    n = dchi.nalldofs()
    # set-up: the regular entry point builds the pattern and gives the reference values
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=precision)
    ref = K.tocsr()
    ref.sort_indices()
    out = torch.empty(K.nnz, dtype=torch.float64, device="cuda:0")  # owned by the caller
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        femm.ctx.call("fs_stiffness_values_noalloc", precision, ctypes.c_int64(n),
                      ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(out.numel()))
        vals = out.cpu().numpy()
        assert np.all(np.isfinite(vals))
        # same CSR order as the regular result (symmetric pattern: CSC == CSR)
        err = np.abs(vals - ref.data).max() / np.abs(ref.data).max()
        assert err <= TOL[precision], err
        # both entry points run the same element and gather kernels: same bits
        assert np.array_equal(vals, ref.data)
    femm.close()


def test_noalloc_rejects_a_beam_mesh():
    # a co-rotational beam context with its pattern built and shell parameters
    # set still has no shell element kernel: rejected before any launch
    import torch
    from flexshell._lib import Context
    xyz = np.asfortranarray([[0.0, 0, 0], [1.0, 0, 0], [2.0, 0, 0]])
    conn = np.ascontiguousarray([[1, 2], [2, 3]], dtype=np.int64)
    dof = np.asfortranarray(np.arange(1, 19, dtype=np.int64).reshape(3, 6))
    ctx = Context(0)
    ctx.call("fs_mesh_set", _abi.FS_COROTBEAM, 3, ptr(xyz), 2, ptr(conn), None, ptr(dof))
    sec = (_abi.fs_beam_section * 2)()
    arr = np.frombuffer(sec, dtype=np.float64).reshape(2, 10)
    arr[:, 0], arr[:, 1], arr[:, 2], arr[:, 3], arr[:, 4] = 0.01, 2e-5, 1e-5, 1e-5, 2e-5
    arr[:, 5], arr[:, 6], arr[:, 9] = np.inf, np.inf, 1.0
    ctx.call("fs_beam_setup", sec, 2.1e11, 0.3, 7850.0)
    nnz = ctypes.c_int64()
    ctx.call("fs_beam_matrix", _abi.FS_BEAM_STIFFNESS, 1, 0, ctypes.c_int64(18), ctypes.byref(nnz))
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    ctx.call("fs_params_set", _abi.make_params(Dps, Dt, 7850.0, 0.01), None)
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_normals_set", ptr(np.zeros((3, 3), order="F")), ptr(np.ones(3, np.uint8)))
    assert ei.value.code == _abi.FS_ERR_UNSUPPORTED
    out = torch.empty(max(nnz.value, 1), dtype=torch.float64, device="cuda:0")
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_stiffness_values_noalloc", _abi.FS_FP64, ctypes.c_int64(18),
                 ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(out.numel()))
    assert ei.value.code == _abi.FS_ERR_UNSUPPORTED
    assert "beam" in str(ei.value)
    ctx.close()


def test_noalloc_rejects_meshes_beyond_the_fixed_scratch():
    import torch
    # 100 x 100 quads -> 20,000 triangles: above the 19,418 FP64 T3FF elements
    # that the 32 MiB array holds, below the 38,836 of the mixed path
    femm, geom0, dchi = _femm(100, False)
    n = dchi.nalldofs()
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    out = torch.empty(K.nnz, dtype=torch.float64, device="cuda:0")
    with pytest.raises(FlexShellError) as ei:
        femm.ctx.call("fs_stiffness_values_noalloc", _abi.FS_FP64, ctypes.c_int64(n),
                      ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(out.numel()))
    assert ei.value.code == _abi.FS_ERR_UNSUPPORTED
    assert "too large" in str(ei.value)
    femm.ctx.call("fs_stiffness_values_noalloc", _abi.FS_MIXED, ctypes.c_int64(n),
                  ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(out.numel()))
    Km = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=_abi.FS_MIXED).tocsr()
    Km.sort_indices()
    vals = out.cpu().numpy()
    assert np.abs(vals - Km.data).max() <= 1e-6 * np.abs(Km.data).max()
    femm.close()

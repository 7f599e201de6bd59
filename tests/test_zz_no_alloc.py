"""The allocation-free stiffness entry point (fs_stiffness_values_noalloc).

It serves callers that cannot let the library allocate device memory when
they ask for a stiffness (their own pool allocator owns the GPU memory, or
their solver loop runs under a fixed memory budget).  The test calls it
through the C ABI, twice in a row, into a device buffer the caller owns, and
checks the values against the regular fs_stiffness entry point with the
tolerance of the other GPU tests.  This file is collected last so that a run
stopping at the first failure has run every other test before it.
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
    femm.close()


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

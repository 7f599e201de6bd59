"""Shift-invert support for the lowest modes (fs_shift_factor, fs_shift_solve;
flexshell.eigs, the reference's eigs(K_ff, M_ff; nev, which = :SM) of
test/test_composite_shell_dynamics.jl:70-76) against SciPy on the same
matrices.  Tolerances: solves to a relative residual of 1e-10, eigenvalues
within 1e-10 of ARPACK with SciPy's own factorisation; the compensated mixed
stiffness within 1e-6 of FP64 on the 20 lowest eigenvalues of the layered
plate."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

import flexshell as F
from flexshell import _abi
from flexshell._lib import FlexShellError, ptr
import problems as PB

pytestmark = pytest.mark.gpu


def _c4(n, triangles=False):
    xyz, conn, dof, nfree, plies = PB.c4_plate(n)
    g = F.laminate(plies)
    femm = (F.FEMMShellT3FFComp(F.mesh.quads_to_triangles(conn), g) if triangles
            else F.FEMMShellQ4RSComp(conn, g))
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    return femm, geom0, dchi, nfree


def test_factor_and_solve_match_scipy():
    femm, geom0, dchi, nf = _c4(12)
    Md = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nf), geom0, dchi).diagonal()
    K = femm.stiffness(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparse(), nf), geom0, None, None, dchi)
    S = F.ShiftInvert(femm.ctx, Md, -2.0)
    A = (K + 2.0 * sp.diags(Md)).tocsc()
    # the half-bandwidth is that of the stored (structural) pattern
    Kc = K.tocoo()
    assert S.bandwidth == int((Kc.row - Kc.col).max())
    rng = np.random.default_rng(0)
    b = rng.normal(size=nf)
    x = S.solve(b)
    xr = spl.spsolve(A, b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert np.abs(x - xr).max() <= 1e-9 * np.abs(xr).max()
    B = rng.normal(size=(nf, 5))
    X = S.solve(B)
    assert np.linalg.norm(A @ X - B) <= 1e-10 * np.linalg.norm(B)
    femm.close()


def test_eigs_matches_arpack_with_scipy_factor():
    femm, geom0, dchi, nf = _c4(20)
    d, v = F.eigs(femm, geom0, dchi, 10, sigma=-1.0, nfree=nf)
    Md = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nf), geom0, dchi).diagonal()
    K = femm.stiffness(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparse(), nf), geom0, None, None, dchi)
    w = np.sort(spl.eigsh(K.tocsc(), k=10, M=sp.diags(Md).tocsc(), sigma=-1.0, which="LM",
                          return_eigenvectors=False, tol=0.0))
    assert np.abs(d - w).max() <= 1e-10 * np.abs(w).max()
    # eigenvectors: K v = d M v
    r = K @ v - (Md[:, None] * v) * d[None, :]
    assert np.abs(r).max() <= 1e-8 * np.abs(K @ v).max()
    # which = SM (shift 0), as Arpack.jl takes it
    d0 = F.eigs(femm, geom0, dchi, 4, nfree=nf, return_eigenvectors=False)
    assert np.abs(d0 - w[:4]).max() <= 1e-10 * np.abs(w[:4]).max()
    femm.close()


@pytest.mark.parametrize("triangles", [False, True])
def test_mixed_comp_lowest_eigenvalues_within_1e6(triangles):
    # the layered plate as Q4RSComp (three-level compensated element sums) and
    # with its quads split as T3FFComp (Dot2)
    femm, geom0, dchi, nf = _c4(48, triangles)
    d64 = F.eigs(femm, geom0, dchi, 20, sigma=-1.0, nfree=nf, return_eigenvectors=False)
    dc = F.eigs(femm, geom0, dchi, 20, sigma=-1.0, nfree=nf, precision=F.FS_MIXED_COMP,
                return_eigenvectors=False)
    assert (np.abs(dc - d64) / np.abs(d64)).max() <= 1e-6
    femm.close()


def test_shift_errors():
    femm, geom0, dchi, nf = _c4(6)
    with pytest.raises(FlexShellError) as ei:
        femm.ctx.call("fs_shift_solve", 1, ptr(np.zeros(nf)), ptr(np.zeros(nf)))
    assert ei.value.code == _abi.FS_ERR_STATE
    Md = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nf), geom0, dchi).diagonal()
    # the last matrix is the mass, not a stiffness
    with pytest.raises(FlexShellError) as ei:
        F.ShiftInvert(femm.ctx, Md, 0.0)
    assert ei.value.code == _abi.FS_ERR_STATE
    K = femm.stiffness(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparse(), nf), geom0, None, None, dchi)
    # a shift above the lowest eigenvalue: K - sigma M is indefinite
    w0 = spl.eigsh(K.tocsc(), k=1, M=sp.diags(Md).tocsc(), sigma=-1.0, which="LM", return_eigenvectors=False)[0]
    with pytest.raises(FlexShellError) as ei:
        F.ShiftInvert(femm.ctx, Md, 2.0 * w0)
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    assert "positive definite" in str(ei.value)
    # a new dof numbering releases the factor: the next solve is refused
    # instead of using a factor whose size and band belong to the old one
    femm.stiffness(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparse(), nf), geom0, None, None, dchi)
    S = F.ShiftInvert(femm.ctx, Md, -1.0)
    S.solve(np.ones(nf))
    femm.ctx.call("fs_dofs_set", ptr(np.asfortranarray(dchi.dofnums, dtype=np.int64)))
    with pytest.raises(FlexShellError) as ei:
        S.solve(np.ones(nf))
    assert ei.value.code == _abi.FS_ERR_STATE
    femm.close()

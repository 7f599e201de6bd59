"""Lowest modes of a shell model with the factorisation on the GPU.

The reference computes free vibration modes with Arpack.jl

    d, v, nconv = eigs(Symmetric(K_ff), Symmetric(M_ff); nev = neigvs, which = :SM)

(test/test_composite_shell_dynamics.jl:70-76, test/test_shell_dynamics.jl:79-80):
ARPACK in shift-invert mode, each iteration a solve with K - sigma M.  `eigs`
below is that call: the free-free stiffness and the lumped mass are assembled
by the library, K - sigma M is factorised on the GPU (fs_shift_factor: banded
Cholesky, double) and ARPACK (SciPy's eigsh, the same library) runs with
solves on the GPU (fs_shift_solve).  which = "SM" is the shift 0, as
Arpack.jl takes it.
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import ptr
from .femm import SysmatAssemblerFFBlock, SysmatAssemblerSparse, SysmatAssemblerSparseDiag


class ShiftInvert:
    """(K - sigma M)^{-1} for the last stiffness assembled in `ctx` and a
    diagonal mass: a scipy LinearOperator for ARPACK's OPinv."""

    def __init__(self, ctx, mdiag, sigma):
        self.ctx = ctx
        self.mdiag = np.ascontiguousarray(mdiag, dtype=np.float64)
        self.n = self.mdiag.shape[0]
        self.sigma = float(sigma)
        kd = ctypes.c_int64()
        ctx.call("fs_shift_factor", ctypes.c_double(self.sigma), ptr(self.mdiag), ctypes.byref(kd))
        self.bandwidth = kd.value

    def solve(self, b):
        b = np.asarray(b, dtype=np.float64)
        one = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.n, -1))
        X = np.empty_like(B, order="F")
        self.ctx.call("fs_shift_solve", int(B.shape[1]), ptr(B), ptr(X))
        return X[:, 0] if one else X

    def operator(self):
        import scipy.sparse.linalg as spl
        return spl.LinearOperator((self.n, self.n), matvec=self.solve, matmat=self.solve, dtype=np.float64)


def eigs(femm, geom0, dchi, nev, which="SM", sigma=None, precision=_abi.FS_FP64, tol=0.0,
         return_eigenvectors=True, nfree=None):
    """The nev eigenvalues (and vectors) of (K_ff, M_ff) nearest the shift
    (which "SM": sigma 0), K the shell stiffness in the given arithmetic and
    M the lumped mass, both the free-free blocks of dchi's numbering (nfree
    free dofs; default dchi.nfreedofs).  Returns (d ascending, v) or d."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    if which != "SM" and sigma is None:
        raise ValueError("only the modes nearest a shift: which = 'SM' or a sigma")
    s = 0.0 if sigma is None else float(sigma)
    nf = int(nfree) if nfree is not None else int(dchi.nfreedofs)
    if nf <= 0:
        raise ValueError("no free dofs: number the dofs (numberdofs) or pass nfree")
    # the mass first: the factorisation takes the last matrix assembled, the stiffness
    Md = femm.mass(SysmatAssemblerFFBlock(SysmatAssemblerSparseDiag(), nf), geom0, dchi).diagonal()
    K = femm.stiffness(SysmatAssemblerFFBlock(SysmatAssemblerSparse(), nf), geom0, None, None, dchi,
                       precision=precision)
    op = ShiftInvert(femm.ctx, Md, s).operator()
    M = sp.diags(Md).tocsc()
    res = spl.eigsh(K, k=nev, M=M, sigma=s, which="LM", OPinv=op, tol=tol,
                    return_eigenvectors=return_eigenvectors)
    if not return_eigenvectors:
        return np.sort(res)
    d, v = res
    o = np.argsort(d)
    return d[o], v[:, o]

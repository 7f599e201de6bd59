"""The reference-facing mirror through the C ABI, on the GPU: the
SysmatAssemblerSparseCSRSymm result type (src/AssemblyModule.jl:47-53), the
shells' restoring force of the layered FEMMs, a per-element thickness (the
otherdimension of every element, src/FEMMShellT3FFModule.jl:677), and the
central-difference loop in the compensated mode.  Tolerances: FP64 1e-12
relative to the largest value, the compensated loop 1e-7."""
import numpy as np
import pytest
import scipy.sparse as sp

import flexshell as F
from flexshell import materials
from oracle import oracle as O
import problems as PB
from checks import relmax, same_pattern

pytestmark = pytest.mark.gpu
STEEL = materials.MatDeforElastIso(200e9, 0.3, 7850.0)


def _homog(quads, thickness, n=10):
    xyz, conn, dof, nfree = PB.jittered_plate(n, quads, wavy=0.02, seed=7)
    femm = (F.FEMMShellQ4RS if quads else F.FEMMShellT3FF)(conn, thickness, STEEL)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    return femm, geom0, dchi, xyz, conn, dof, nfree


@pytest.mark.parametrize("quads", [False, True])
def test_csr_assembler_returns_the_csr_of_the_same_matrix(quads):
    femm, geom0, dchi, *_ = _homog(quads, 0.01)
    Kc = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Kr = femm.stiffness(F.SysmatAssemblerSparseCSRSymm(), geom0, None, None, dchi)
    assert sp.isspmatrix_csr(Kr) and sp.isspmatrix_csc(Kc)
    # the symmetric matrix: the CSC arrays are the CSR arrays
    assert np.array_equal(Kr.indptr, Kc.indptr) and np.array_equal(Kr.indices, Kc.indices)
    assert np.array_equal(Kr.data, Kc.data)
    assert abs(Kr - Kc).max() == 0.0
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_per_element_thickness_matches_oracle(quads):
    xyz, conn, dof, nfree = PB.jittered_plate(10, quads, wavy=0.02, seed=7)
    t = 0.005 + 0.01 * np.random.default_rng(3).random(conn.shape[0])
    femm, geom0, dchi, *_ = _homog(quads, t)
    Dps, Dt = materials.shell_material_stiffness(STEEL)
    P = O.Problem(O.Q4RS if quads else O.T3FF, xyz, conn, dof, thickness=t,
                  material=dict(Dps=Dps, Dt=Dt, rho=7850.0))
    P.compute_normals()
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert same_pattern(K, Ko) and relmax(K, Ko) <= 1e-12
    M = femm.mass(F.SysmatAssemblerSparseSymm(), geom0, dchi)
    assert relmax(M, P.assemble_scipy("M", O.DROP_ZEROS)) <= 1e-12
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_layered_restoring_force_is_minus_K_U(quads):
    xyz, conn, dof, nfree = PB.jittered_plate(8, quads, wavy=0.02, seed=9)
    g = F.laminate(PB.cross_ply_groups((0, 45, -45, 90)))
    femm = (F.FEMMShellQ4RSComp if quads else F.FEMMShellT3FFComp)(conn, g)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.random.default_rng(1).normal(size=(xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    Fr = femm.restoringforce(geom0, None, None, dchi)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    n = dchi.nalldofs()
    U = np.zeros(n)
    U[dof.ravel(order="F") - 1] = dchi.values.ravel(order="F")
    ref = -(K @ U)
    assert np.abs(Fr - ref).max() <= 1e-12 * np.abs(ref).max()
    femm.close()


def test_cd_loop_compensated_follows_fp64():
    femm, geom0, dchi, xyz, conn, dof, nfree = _homog(True, 0.01, n=16)
    m = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi).diagonal()
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    import ctypes
    from flexshell._lib import ptr
    om = ctypes.c_double()
    femm.ctx.call("fs_power_iteration", ptr(np.ascontiguousarray(m)), ctypes.c_int64(300), ctypes.c_uint64(3),
                  ctypes.byref(om))
    dt = 0.9 * 2 / om.value
    V0 = np.zeros(nfree)
    wd = dof[:, 2]
    fw = wd <= nfree
    V0[wd[fw] - 1] = 1e-3 * np.sin(np.pi * xyz[fw, 0]) * np.sin(np.pi * xyz[fw, 1])
    res = {}
    for prec in (F.FS_FP64, F.FS_MIXED_COMP):
        U, V, A = F.cd_loop(femm, m, 0.02, om.value / 10, np.zeros(nfree), V0, 400 * dt, dt,
                            peek_every=100, precision=prec)
        res[prec] = U
    err = np.abs(res[F.FS_MIXED_COMP] - res[F.FS_FP64]).max() / np.abs(res[F.FS_FP64]).max()
    assert err <= 1e-7, err
    femm.close()


def test_inputs_changed_in_place_are_uploaded():
    # the reference reads geom0 and dchi on every call: nodes moved in place
    # and dofs renumbered in place (the same array objects) reach the next
    # stiffness, which equals a fresh FEMM's on the same inputs (with the
    # first FEMM's normals: neither recomputes them without associategeometry)
    femm, geom0, dchi, xyz, conn, dof, nfree = _homog(False, 0.01, n=6)
    K0 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    geom0.values[:, 2] += 0.05 * geom0.values[:, 0] ** 2
    dchi.dofnums[[0, 1]] = dchi.dofnums[[1, 0]]
    K1 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    fresh = F.FEMMShellT3FF(conn, 0.01, STEEL)
    g2 = F.NodalField(np.array(geom0.values))
    d2 = F.NodalField(np.zeros((xyz.shape[0], 6)))
    d2.dofnums = np.asfortranarray(np.array(dchi.dofnums))
    fresh.associategeometry(g2)
    fresh.set_normals(femm._normals, femm._normal_valid)
    Kf = fresh.stiffness(F.SysmatAssemblerSparse(), g2, None, None, d2)
    assert abs(K1 - K0).max() > 0
    assert same_pattern(K1, Kf) and np.array_equal(K1.tocsc().data, Kf.tocsc().data)
    fresh.close()
    femm.close()

"""GPU parity on the reference configurations themselves, through the C ABI.

Configuration 1: a flat 1 m x 1 m plate, 32 x 32 quads each split into two
T3FF triangles (2,048 elements, 1,089 nodes), interior nodes jittered
U(+-0.2 h) in plane from a seed, thickness 0.01 m, steel (E 200 GPa,
nu 0.3, rho 7850 kg/m^3), the edge x = 0 clamped: FP64 stiffness and lumped
mass against the oracle (src/FEMMShellT3FFModule.jl:635-736, :757-811).

Configuration 2 at 256 x 256 quads (the full 1024 x 1024 plate is checked
against the oracle by the benchmark): the jittered plate with
z = 0.01 sin(pi x) sin(pi y), thickness 0.005 m, as T3FF (131,072
triangles) and Q4RS (65,536 quads, src/FEMMShellQ4RSModule.jl:877-947).

Tolerances (written here): FP64 -- identical pattern, max |dK| / max |K| and
max |dK_ij| / sqrt(|K_ii K_jj|) (every entry against its own scale) at most
1e-12, and the relative error of every entry above 1e-12 max |K| at most
1e-5.  The last is a cancellation measure, not an accuracy bar: an entry
1e-12 of the largest is summed from terms of the size of its row's diagonal
and carries their rounding (measured on the GPU: 1.9e-9 for T3FF at 256^2,
1.1e-8 for T3FF and 1.2e-6 for Q4RS at 1024^2, while the scaled error there
was 1.5e-15 and 1.5e-13); mixed paths -- at most 1e-6 in max |dK| / max |K|.
"""
import numpy as np
import pytest

import flexshell as F
from flexshell import materials
from oracle import oracle as O
import problems as PB
from checks import entrywise_errors, relmax, same_pattern, same_pattern_modulo_cancellation

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
ENTRY_TOL = 1e-5
MIXED_TOL = 1e-6
STEEL = materials.MatDeforElastIso(200e9, 0.3, 7850.0)


def _pair(xyz, conn, dof, thickness, quads):
    Dps, Dt = materials.shell_material_stiffness(STEEL)
    P = O.Problem(O.Q4RS if quads else O.T3FF, xyz, conn, dof, thickness=thickness,
                  material=dict(Dps=Dps, Dt=Dt, rho=7850.0))
    P.compute_normals()
    femm = (F.FEMMShellQ4RS if quads else F.FEMMShellT3FF)(conn, thickness, STEEL)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    assert np.allclose(femm._normals, P.normals, rtol=0, atol=1e-14)
    assert np.array_equal(femm._normal_valid, P.valid)
    return P, femm, geom0, dchi


def _fp64_checks(K, Ko):
    assert same_pattern(K, Ko)
    e = entrywise_errors(K, Ko)
    assert e["relmax"] <= FP64_TOL, e
    assert e["scaled"] <= FP64_TOL, e
    assert e["entrywise"] <= ENTRY_TOL, e
    return e


def test_config1_t3ff_32x32_clamped_fp64_k_and_lumped_m():
    xyz, conn, dof, nfree = PB.jittered_plate(32, False, jitter=0.2, seed=0)
    assert conn.shape[0] == 2048 and xyz.shape[0] == 1089
    P, femm, geom0, dchi = _pair(xyz, conn, dof, 0.01, False)
    nall = dchi.nalldofs()
    assert nall == 6534
    # all dofs (SysmatAssemblerSparse): the structural pattern of the survey, 264,996 entries
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert K.nnz == 264996
    _fp64_checks(K, Ko)
    # the default assembler (zeros dropped) and the free-free block
    Ks = femm.stiffness(F.SysmatAssemblerSparseSymm(), geom0, None, None, dchi)
    Kso = P.assemble_scipy("K", O.DROP_ZEROS)
    assert same_pattern_modulo_cancellation(Ks, Kso)
    assert relmax(Ks, Kso) <= FP64_TOL
    Kf = femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    _fp64_checks(Kf, P.assemble_scipy("K", O.KEEP_ZEROS, n=nfree))
    # lumped mass, both structural assemblers
    for asm, mode in ((F.SysmatAssemblerSparse(), O.KEEP_ZEROS), (F.SysmatAssemblerSparseSymm(), O.DROP_ZEROS)):
        M = femm.mass(asm, geom0, dchi)
        Mo = P.assemble_scipy("M", mode)
        assert same_pattern(M, Mo)
        assert relmax(M, Mo) <= FP64_TOL
    # total translational mass rho t A in each direction
    Md = femm.mass(F.SysmatAssemblerSparseDiag(), geom0, dchi).diagonal()
    ux = dof[:, 0] - 1
    assert abs(Md[ux].sum() - 7850.0 * 0.01 * 1.0) <= 1e-12 * 78.5
    # mixed precisions against the oracle
    for prec in (F.FS_MIXED, F.FS_MIXED_COMP):
        Km = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=prec)
        assert same_pattern(Km, Ko)
        assert relmax(Km, Ko) <= MIXED_TOL
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_config2_plate_256_fp64_vs_oracle(quads):
    xyz, conn, dof, nfree = PB.jittered_plate(256, quads, jitter=0.2, seed=0, wavy=0.01, clamp_x0=False)
    P, femm, geom0, dchi = _pair(xyz, conn, dof, 0.005, quads)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    e = _fp64_checks(K, Ko)
    # the pattern-accumulating oracle helper used at the full size agrees
    Kc = K.tocsc()
    vals, touched, missing = P.stiffness_into_pattern(Kc.indptr + 1, Kc.indices + 1)
    assert missing == 0 and touched.all()
    assert np.abs(vals - Kc.data).max() <= FP64_TOL * np.abs(Kc.data).max()
    M = femm.mass(F.SysmatAssemblerSparseDiag(), geom0, dchi)
    Mo = P.assemble_scipy("M", O.DIAG)
    assert relmax(M, Mo) <= FP64_TOL
    for prec in (F.FS_MIXED, F.FS_MIXED_COMP):
        Km = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=prec)
        assert same_pattern(Km, Ko)
        assert relmax(Km, Ko) <= MIXED_TOL
    femm.close()
    assert e["relmax"] <= FP64_TOL

"""GPU parity of the co-rotational beam kernels (FEMMCorotBeam) against the
oracle, through the C ABI, and the reference's beam known answers run on the
GPU.  Tolerance: 1e-12 relative (max-abs difference over max-abs value) for
element matrices, assembled matrices and vectors; identical sparsity pattern
for the pattern-keeping assembler."""
import ctypes

import numpy as np
import pytest

from flexshell import _abi, beam as B
from flexshell.femm import (NodalField, SysmatAssemblerFFBlock, SysmatAssemblerSparse,
                            SysmatAssemblerSparseDiag, SysmatAssemblerSparseSymm)
from flexshell._lib import FlexShellError
from oracle import oracle as O
import beams as BM
from checks import relmax, same_pattern, same_pattern_modulo_cancellation

pytestmark = pytest.mark.gpu

TOL = 1e-12
MATS = [(_abi.FS_BEAM_STIFFNESS, O.BEAM_STIFFNESS), (_abi.FS_BEAM_GEOSTIFFNESS, O.BEAM_GEOSTIFFNESS),
        (_abi.FS_BEAM_MASS, O.BEAM_MASS), (_abi.FS_BEAM_GYROSCOPIC, O.BEAM_GYROSCOPIC)]


@pytest.fixture(scope="module")
def frame():
    xyz, conn, sec, u1, R1, v1, dof, nf = BM.lattice_frame()
    mat = BM.Material(2.1e3, 0.3, 7.8)
    femm = B.FEMMCorotBeam(conn, sec, mat)
    orc = O.Beam(xyz, conn, sec, mat.E, mat.nu, mat.rho)
    geom0 = NodalField(xyz)
    dchi = NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    dchi.nfreedofs = nf
    yield dict(femm=femm, orc=orc, geom0=geom0, dchi=dchi, u1=u1, R1=R1, v1=v1, dof=dof, nf=nf,
               conn=conn, xyz=xyz)
    femm.close()


def _elem_err(G, R, floor=None):
    """max over elements of max|G - R| / max|R|; `floor` (per element) replaces
    max|R| where the exact result is zero and both sides are round-off."""
    errs = []
    for k, (g, r) in enumerate(zip(G, R)):
        scale = np.abs(r).max()
        if floor is not None:
            scale = max(scale, floor[k])
        errs.append(np.abs(g - r).max() / max(scale, 1e-300))
    return max(errs)


@pytest.mark.parametrize("which", range(4))
@pytest.mark.parametrize("mass_type", range(4))
def test_element_matrices_match_oracle(frame, which, mass_type):
    if which in (0, 1) and mass_type:
        pytest.skip("mass_type only changes the mass and gyroscopic matrices")
    f = frame
    fw, ow = MATS[which]
    G = f["femm"].element_matrices(fw, f["geom0"], f["u1"], f["R1"], f["v1"], mass_type=mass_type)
    R = f["orc"].elements(ow, u1=f["u1"], R1=f["R1"], v1=f["v1"], mass_type=mass_type)
    floor = None
    if which == 3:
        # OS M - M OS vanishes for an isotropic (lumped translational) mass:
        # measure it against |M| |v| instead of its own round-off
        Mo = f["orc"].elements(O.BEAM_MASS, u1=f["u1"], R1=f["R1"], mass_type=mass_type)
        floor = [np.abs(m).max() * np.abs(f["v1"]).max() for m in Mo]
    assert _elem_err(G, R, floor) <= TOL
    assert np.abs(G - G.transpose(0, 2, 1)).max() <= 1e-13 * np.abs(G).max()


def test_element_vectors_match_oracle(frame):
    f = frame
    G = f["femm"].element_vectors(_abi.FS_BEAM_RESTORING, f["geom0"], f["u1"], f["R1"])
    R = f["orc"].elements(O.BEAM_RESTORING, u1=f["u1"], R1=f["R1"])
    assert _elem_err(G, R) <= TOL
    q = np.random.default_rng(5).normal(size=(f["conn"].shape[0], 3))
    G = f["femm"].element_vectors(_abi.FS_BEAM_DISTRIBLOAD, f["geom0"], f["u1"], f["R1"], q=q)
    R = f["orc"].elements(O.BEAM_DISTRIBLOAD, u1=f["u1"], R1=f["R1"], q=q)
    assert _elem_err(G, R) <= TOL


@pytest.mark.parametrize("which", range(4))
def test_assembled_matrices_match_oracle(frame, which):
    f = frame
    fw, ow = MATS[which]
    n = f["dchi"].nalldofs()
    calls = {0: "stiffness", 1: "geostiffness", 2: "mass", 3: "gyroscopic"}
    femm = f["femm"]

    def gpu(asm):
        args = (asm, f["geom0"], f["u1"], f["R1"]) + ((f["v1"],) if which == 3 else ()) + (f["dchi"],)
        return getattr(femm, calls[which])(*args)

    kw = dict(u1=f["u1"], R1=f["R1"], v1=f["v1"])
    # pattern-keeping assembler: identical pattern, values within TOL
    A = gpu(SysmatAssemblerSparse())
    Ro = f["orc"].matrix(ow, f["dof"], n, mode=O.KEEP_ZEROS, **kw)
    assert same_pattern(A, Ro) and relmax(A, Ro) <= TOL
    # default assembler (zero entries dropped)
    A = gpu(SysmatAssemblerSparseSymm())
    Ro = f["orc"].matrix(ow, f["dof"], n, mode=O.DROP_ZEROS, **kw)
    assert same_pattern_modulo_cancellation(A, Ro) and relmax(A, Ro) <= TOL
    # free-free block
    nf = f["nf"]
    A = gpu(SysmatAssemblerFFBlock(SysmatAssemblerSparse(), nf))
    Ro = f["orc"].matrix(ow, f["dof"], nf, mode=O.KEEP_ZEROS, **kw)
    assert same_pattern(A, Ro) and relmax(A, Ro) <= TOL
    # diagonal
    A = gpu(SysmatAssemblerSparseDiag())
    Ro = f["orc"].matrix(ow, f["dof"], n, mode=O.DIAG, **kw)
    assert np.abs(A.diagonal() - Ro.diagonal()).max() <= TOL * np.abs(Ro.diagonal()).max()


def test_assembled_vectors_match_oracle(frame):
    f = frame
    n = f["dchi"].nalldofs()
    F = f["femm"].restoringforce(f["geom0"], f["u1"], f["R1"], f["dchi"])
    R = f["orc"].vector(O.BEAM_RESTORING, f["dof"], n, u1=f["u1"], R1=f["R1"])
    assert np.abs(F - R).max() <= TOL * np.abs(R).max()
    q = [0.3, -1.0, 2.0]
    F = f["femm"].distribloads_global(f["geom0"], f["u1"], f["R1"], f["dchi"], q)
    R = f["orc"].vector(O.BEAM_DISTRIBLOAD, f["dof"], n, u1=f["u1"], R1=f["R1"], q=q)
    assert np.abs(F - R).max() <= TOL * np.abs(R).max()


def test_reference_lframe_frequencies_on_gpu():
    f, eng = BM.lframe_modal(BM.GpuBeams)
    eng.close()
    fo, _ = BM.lframe_modal(BM.OracleBeams)
    assert np.linalg.norm(f - BM.LFRAME_FREQS) / np.linalg.norm(BM.LFRAME_FREQS) <= 3.0e-5
    assert np.abs(f - fo).max() <= 1e-10 * fo.max()


def test_reference_buckling_factors_on_gpu():
    fs, eng = BM.cantilever_buckling(BM.GpuBeams)
    eng.close()
    assert np.linalg.norm(fs - BM.BUCKLING_FACTORS) / np.linalg.norm(BM.BUCKLING_FACTORS) <= 1.0e-3
    fo, _ = BM.cantilever_buckling(BM.OracleBeams)
    assert np.abs(fs - fo).max() <= 1e-8 * fo.max()


def test_reference_fast_top_on_gpu():
    x, y, eng = BM.fast_top(BM.GpuBeams)
    eng.close()
    assert np.linalg.norm(x - BM.FAST_TOP_TIPX) / np.linalg.norm(BM.FAST_TOP_TIPX) <= 1.0e-3
    assert np.linalg.norm(y - BM.FAST_TOP_TIPY) / np.linalg.norm(BM.FAST_TOP_TIPY) <= 1.0e-3


def test_beam_errors(frame):
    f = frame
    femm = B.FEMMCorotBeam(f["conn"], np.zeros((f["conn"].shape[0], 10)), BM.Material(1.0, 0.3))
    with pytest.raises(FlexShellError) as ei:
        femm.stiffness(f["geom0"], f["u1"], f["R1"], f["dchi"])  # zero areas rejected at set-up
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    femm.close()
    # shell entry points refuse a beam mesh
    ctx = f["femm"].ctx
    nnz = ctypes.c_int64()
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_stiffness", _abi.FS_FP64, _abi.FS_ASM_SPARSE, f["dchi"].nalldofs(), ctypes.byref(nnz))
    assert ei.value.code == _abi.FS_ERR_UNSUPPORTED
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_beam_matrix", 7, 0, _abi.FS_ASM_SPARSE, 10, ctypes.byref(nnz))
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT

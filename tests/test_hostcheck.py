"""The CUDA library's per-element math, built for the host, against the oracle.

The library rewrites the reference's dense congruences as a Gram product of
strain rows on the global dofs (csrc/fs_elem_math.cuh).  This CPU test runs
that exact header on the host (tests/hostcheck) and compares every element
matrix with the oracle's dense restatement, so the formulation is checked
before any GPU run.  The GPU parity tests then check the kernels themselves.
"""
import numpy as np
import pytest

from oracle import oracle as O
from flexshell import _abi
import problems as PB
from hostcheck import hostmath as HC


def _homog(quads, n=4, tsf=0, crease=False):
    d = PB.scordelis_lo(quads, n)
    et = O.Q4RS if quads else O.T3FF
    P = O.Problem(et, d["xyz"], d["conn"], d["dofnums"], thickness=d["thickness"],
                  material=d["material"], stab_c=d["stab_c"], tsf=tsf)
    P.compute_normals()
    if crease:
        v = P.valid.copy()
        v[::3] = 0
        P.set_normals(P.normals, v)
    prm = _abi.make_params(d["material"]["Dps"], d["material"]["Dt"], 0.0, d["thickness"],
                           stab_c=d["stab_c"], transv_shear_formulation=tsf, quads=quads)
    return et, d, P, prm


def _relmax(A, B):
    return np.abs(A - B).max() / np.abs(B).max()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("crease", [False, True])
def test_homogeneous_fp64_matches_oracle(quads, crease):
    et, d, P, prm = _homog(quads, crease=crease)
    Ko = P.element_stiffness()
    Kh = HC.element_matrices(et, _abi.FS_FP64, d["xyz"], d["conn"], P.normals, P.valid,
                             d["thickness"], prm)
    for e in range(len(Ko)):
        assert _relmax(Kh[e], Ko[e]) <= 1e-12


def test_t3_average_k_fp64_matches_oracle():
    et, d, P, prm = _homog(False, tsf=1)
    Ko = P.element_stiffness()
    Kh = HC.element_matrices(et, _abi.FS_FP64, d["xyz"], d["conn"], P.normals, P.valid,
                             d["thickness"], prm)
    assert max(_relmax(Kh[e], Ko[e]) for e in range(len(Ko))) <= 1e-12


@pytest.mark.parametrize("quads", [False, True])
def test_homogeneous_mixed_error(quads):
    et, d, P, prm = _homog(quads)
    Ko = P.element_stiffness()
    Kh = HC.element_matrices(et, _abi.FS_MIXED, d["xyz"], d["conn"], P.normals, P.valid,
                             d["thickness"], prm)
    assert _relmax(Kh, Ko) <= 1e-6


def _composite(quads, n=6, csmat=None, angles=(0, 90, 90, 0)):
    plies = PB.cross_ply_groups(angles)
    A, B, D, H, md, mi = O.laminate(plies)
    cs = np.eye(3) if csmat is None else csmat
    t = sum(p["thickness"] for p in plies)
    xyz, conn, dof, nfree = PB.jittered_plate(n, quads, wavy=0.02, seed=5)
    et = O.Q4RSCOMP if quads else O.T3FFCOMP
    stab_c = 0.1 if quads else 5 / 12 / 1.5
    grp = dict(A=A, B=B, D=D, H=H, csmat=cs, thickness=t, mass=md, moi=mi)
    P = O.Problem(et, xyz, conn, dof, groups=[grp], stab_c=stab_c)
    P.compute_normals()
    g = _abi.make_group(A, B, D, H, cs, t, md, mi)
    prm = _abi.make_params(np.eye(3), np.eye(2), 0.0, t, stab_c=stab_c, quads=quads)
    return et, xyz, conn, P, prm, g


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("angles", [(0, 90, 90, 0), (30, -45, 60)])
def test_composite_fp64_matches_oracle(quads, angles):
    c = np.cos(0.3); s = np.sin(0.3)
    cs = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    et, xyz, conn, P, prm, g = _composite(quads, csmat=cs, angles=angles)
    Ko = P.element_stiffness()
    Kh = HC.element_matrices(et, _abi.FS_FP64, xyz, conn, P.normals, P.valid, 0.0, prm,
                             groups=[g], egroup=np.zeros(len(conn)))
    assert max(_relmax(Kh[e], Ko[e]) for e in range(len(Ko))) <= 1e-12


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("angles", [(0, 90, 90, 0), (30, -45, 60)])
@pytest.mark.parametrize("precision", [_abi.FS_MIXED, _abi.FS_MIXED_COMP])
def test_composite_mixed_within_1e6_of_oracle(quads, angles, precision):
    # the layered elements' float rows (rotated layup csys, B != 0) in both
    # mixed modes: every element matrix within 1e-6 of the oracle's FP64 one
    # (measured up to 7.3e-7 with FS_MIXED, 3.9e-7 compensated)
    c = np.cos(0.3); s = np.sin(0.3)
    cs = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    et, xyz, conn, P, prm, g = _composite(quads, csmat=cs, angles=angles)
    Ko = P.element_stiffness()
    Kh = HC.element_matrices(et, precision, xyz, conn, P.normals, P.valid, 0.0, prm,
                             groups=[g], egroup=np.zeros(len(conn)))
    assert max(_relmax(Kh[e], Ko[e]) for e in range(len(Ko))) <= 1e-6


def _beam_case(seed=0):
    import beams
    return beams.lattice_frame(seed=seed)


@pytest.mark.parametrize("which,mass_type", [(0, 1), (1, 1), (2, 0), (2, 1), (2, 2), (2, 3),
                                             (3, 0), (3, 1), (3, 3), (4, 1), (5, 1)])
def test_beam_math_matches_oracle(which, mass_type):
    # the beam kernels' per-element math (csrc/fs_beam_math.cuh: Gram form of
    # aN' DN aN, sub-block rotations) against the oracle's dense Te SM Te'
    xyz, conn, sec, u1, R1, v1, dof, nf = _beam_case()
    E, nu, rho = 2.1e3, 0.3, 7.8
    q = np.random.default_rng(2).normal(size=(conn.shape[0], 3))
    H = HC.beam_elements(which, xyz, conn, sec, E, nu, rho, u1, R1, v1, mass_type, q)
    b = O.Beam(xyz, conn, sec, E, nu, rho)
    R = b.elements(which, u1=u1, R1=R1, v1=v1, mass_type=mass_type, q=q)
    err = max(np.abs(h - r).max() / max(np.abs(r).max(), 1e-300) for h, r in zip(H, R))
    assert err <= 1e-12


def test_q4_basis_at_gauss_points_is_the_computed_basis():
    # the tabulated Q4 basis gradients at the four Gauss points are bitwise
    # the computed ones (q4_dbasis_gp against q4_dbasis)
    gp = HC.q4_basis_pair()
    assert np.array_equal(gp[0], gp[1])

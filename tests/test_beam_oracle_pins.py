"""Pins of the beam oracle (FEMMCorotBeam) against the reference's own known
answers, plus the host-side set-up helpers of flexshell.beam.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from flexshell import beam as B
import beams as BM


def _relnorm(a, ref):
    a, ref = np.asarray(a), np.asarray(ref)
    return np.linalg.norm(a - ref) / np.linalg.norm(ref)


def test_lframe_frequencies():
    # test/test_beam_modal.jl:74: norm(reffs - fs)/norm(reffs) <= 3e-5
    f, _ = BM.lframe_modal(BM.OracleBeams)
    assert _relnorm(f, BM.LFRAME_FREQS) <= 3.0e-5


def test_cantilever_buckling_factors():
    # test/test_beam_buckling.jl:85: rtol 1e-3 on the 2nd and 3rd factors
    fs, _ = BM.cantilever_buckling(BM.OracleBeams)
    assert _relnorm(fs, BM.BUCKLING_FACTORS) <= 1.0e-3


def test_fast_top_trajectory():
    # test/test_beam_dyn.jl:252-253: rtol 1e-3 on the recorded tip coordinates
    x, y, _ = BM.fast_top(BM.OracleBeams)
    assert x.size == len(BM.FAST_TOP_TIPX)
    assert _relnorm(x, BM.FAST_TOP_TIPX) <= 1.0e-3
    assert _relnorm(y, BM.FAST_TOP_TIPY) <= 1.0e-3


def _dense_mass(A, I1, I2, I3, rho, L, mass_type):
    """The dense matrices of local_mass_original! (src/FEMMCorotBeamModule.jl:556-670)."""
    if mass_type >= 2:
        d = np.zeros(12)
        d[[0, 1, 2, 6, 7, 8]] = A * rho * L / 2.0
        if mass_type == 3:
            d[[3, 9]] = rho * I1 * L / 2.0
            d[[4, 10]] = rho * I2 * L / 2.0
            d[[5, 11]] = rho * I3 * L / 2.0
        return np.diag(d)
    a, b = 11 * L / 210, 13 * L / 420
    MM = np.array([
        [1 / 3, 0, 0, 0, 0, 0, 1 / 6, 0, 0, 0, 0, 0],
        [0, 13 / 35, 0, 0, 0, a, 0, 9 / 70, 0, 0, 0, -b],
        [0, 0, 13 / 35, 0, -a, 0, 0, 0, 9 / 70, 0, b, 0],
        [0, 0, 0, I1 / 3 / A, 0, 0, 0, 0, 0, I1 / 6 / A, 0, 0],
        [0, 0, -a, 0, L ** 2 / 105, 0, 0, 0, -b, 0, -L ** 2 / 140, 0],
        [0, a, 0, 0, 0, L ** 2 / 105, 0, b, 0, 0, 0, -L ** 2 / 140],
        [1 / 6, 0, 0, 0, 0, 0, 1 / 3, 0, 0, 0, 0, 0],
        [0, 9 / 70, 0, 0, 0, b, 0, 13 / 35, 0, 0, 0, -a],
        [0, 0, 9 / 70, 0, -b, 0, 0, 0, 13 / 35, 0, a, 0],
        [0, 0, 0, I1 / 6 / A, 0, 0, 0, 0, 0, I1 / 3 / A, 0, 0],
        [0, 0, b, 0, -L ** 2 / 140, 0, 0, 0, a, 0, L ** 2 / 105, 0],
        [0, -b, 0, 0, 0, -L ** 2 / 140, 0, -a, 0, 0, 0, L ** 2 / 105]]) * (rho * A * L)
    if mass_type == 1:
        c, e = L / 10, L ** 2
        MM = MM + (rho / L) * np.array([
            [0] * 12,
            [0, 6 / 5 * I2, 0, 0, 0, c * I2, 0, -6 / 5 * I2, 0, 0, 0, c * I2],
            [0, 0, 6 / 5 * I3, 0, -c * I3, 0, 0, 0, -6 / 5 * I3, 0, -c * I3, 0],
            [0] * 12,
            [0, 0, -c * I3, 0, 2 * e / 15 * I3, 0, 0, 0, c * I3, 0, -e / 30 * I3, 0],
            [0, c * I2, 0, 0, 0, 2 * e / 15 * I2, 0, -c * I2, 0, 0, 0, -e / 30 * I2],
            [0] * 12,
            [0, -6 / 5 * I2, 0, 0, 0, -c * I2, 0, 6 / 5 * I2, 0, 0, 0, -c * I2],
            [0, 0, -6 / 5 * I3, 0, c * I3, 0, 0, 0, 6 / 5 * I3, 0, c * I3, 0],
            [0] * 12,
            [0, 0, -c * I3, 0, -e / 30 * I3, 0, 0, 0, c * I3, 0, 2 * e / 15 * I3, 0],
            [0, c * I2, 0, 0, 0, -e / 30 * I2, 0, -c * I2, 0, 0, 0, 2 * e / 15 * I2]])
    return MM


@pytest.mark.parametrize("mass_type", range(4))
def test_local_mass_formulations(mass_type):
    # test/test_beam_modal.jl:182-196 (and the three modules after it): the
    # element-frame mass equals the dense "original" form to 1e-6
    A, I1, I2, I3, rho, L = 1.3, 35.1, 32.3, 16.5, 10000.0, 3.333
    sec = [[A, I1, I2, I3, 1.0, np.inf, np.inf, 0.0, 1.0, 0.0]]  # element frame = global axes
    b = O.Beam([[0, 0, 0], [L, 0, 0]], [[1, 2]], sec, 1.0, 0.3, rho)
    MM = b.elements(O.BEAM_MASS, mass_type=mass_type)[0]
    ref = _dense_mass(A, I1, I2, I3, rho, L, mass_type)
    assert np.linalg.norm(MM - ref) / np.linalg.norm(ref) <= 1.0e-12


@pytest.mark.parametrize("timoshenko", [False, True])
def test_element_stiffness_rigid_body_modes(timoshenko):
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (2, 3))
    A2s = 0.8 if timoshenko else np.inf
    sec = [[1.0, 0.2, 0.1, 0.07, 0.15, A2s, A2s, *rng.uniform(-1, 1, 3)]]
    b = O.Beam(x, [[1, 2]], sec, 2e3, 0.3, 1.0)
    K = b.elements(O.BEAM_STIFFNESS)[0]
    assert np.abs(K - K.T).max() <= 1e-13 * np.abs(K).max()
    w = np.linalg.eigvalsh(K)
    assert np.all(np.abs(w[:6]) <= 1e-10 * w[-1]) and w[6] > 1e-6 * w[-1]


def test_restoring_force_is_zero_undeformed_and_antisymmetric_in_translation():
    xyz, conn, sec, mat, L = BM.lframe()
    b = O.Beam(xyz, conn, sec, mat.E, mat.nu, mat.rho)
    assert np.abs(b.elements(O.BEAM_RESTORING)).max() == 0.0
    # a rigid translation produces no force either
    u = np.tile([1.5, -2.0, 0.5], (xyz.shape[0], 1))
    assert np.abs(b.elements(O.BEAM_RESTORING, u1=u)).max() <= 1e-9


def test_rectangle_torsion_table_matches_fitpack():
    interp = pytest.importorskip("scipy.interpolate")
    tck = interp.splrep(B._RECT_RATIO, B._RECT_COEF, k=3, s=0)
    for r in [1.0, 1.2, 2.0, 3.3, 8.0, 10.0, 15.0, 33.0, 150.0, 1999.0]:
        assert abs(B._rect_torsion(r) - float(interp.splev(r, tck))) <= 1e-14
    assert B._rect_torsion(5000.0) == B._rect_torsion(2000.0)  # bc = "nearest"


def test_frame_member_and_merge():
    cs = B.CrossSectionCircle(lambda s: 2.0, lambda s: [0.0, 0.0, 1.0])
    m1 = B.frame_member([[0, 0, 0], [10, 0, 0]], 5, cs)
    m2 = B.frame_member([[10, 0, 0], [10, 4, 0]], 2, cs)
    xyz, conn, sec = B.merge_members([m1, m2], tolerance=1e-6)
    assert xyz.shape == (8, 3) and conn.shape == (7, 2)
    assert np.allclose(xyz[5], [10, 0, 0]) and conn[5, 0] == 6
    assert np.allclose(sec[:, 0], np.pi * 4)
    assert np.allclose(sec[:, 4], np.pi / 2 * 16) and np.all(np.isinf(sec[:, 5]))
    # curved member: polynomial through three points
    nodes, c3, _ = B.frame_member([[0, 0, 0], [1, 1, 0], [2, 0, 0]], 4, cs)
    assert np.allclose(nodes[0], [0, 0, 0]) and np.allclose(nodes[-1], [2, 0, 0])


def test_update_rotation_field_composes_rotations():
    R = B.initial_Rfield(1)
    f = type("F", (), {})()
    f.values = np.array([[0, 0, 0, 0.3, 0.0, 0.0]])
    B.update_rotation_field(R, f)
    B.update_rotation_field(R, f)
    assert np.allclose(R.values[0].reshape(3, 3, order="F"), B.rotmat3([0.6, 0, 0]), atol=1e-15)

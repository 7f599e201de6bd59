"""Distributed surface loads (FinEtools 8.2.5 distribloads on the shell
element sets: test/test_shell_statics.jl:84-86, plate_expl_examples.jl:196-199):
the oracle's restatement pinned by closed forms and by the Scordelis-Lo load
whose solution the parity tests hold to the reference's published deflection.
CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
import problems as PB


def _areas(xyz, conn):
    X = xyz[conn - 1]
    return 0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), axis=1)


@pytest.mark.parametrize("rule", [1, 3, 6])
def test_uniform_load_on_triangles_is_a_third_of_the_area(rule):
    xyz, conn, dof, _ = PB.jittered_plate(6, False, jitter=0.2, wavy=0.05, seed=2, clamp_x0=False)
    q = np.array([0.3, -0.2, -90.0, 0.01, 0.02, 0.03])
    F = O.distribloads(xyz, conn, dof, rule, 3, q, int(dof.max()))
    A = _areas(xyz, conn)
    ref = np.zeros((xyz.shape[0], 6))
    for e in range(conn.shape[0]):
        for a in conn[e] - 1:
            ref[a] += q * A[e] / 3
    got = F[dof - 1]
    # TriRule(6)'s published weights carry 15 digits
    tol = 1e-14 if rule < 6 else 1e-13
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("order", [1, 2, 3])
def test_uniform_load_on_parallelogram_quads(order):
    # an affine (sheared) grid: every quad is a parallelogram, so each node
    # gets a quarter of the area of each quad around it for any rule
    n = 5
    xs, ys = np.meshgrid(np.linspace(0, 2, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    xyz = np.c_[xs.ravel() + 0.3 * ys.ravel(), ys.ravel(), 0.1 * xs.ravel()]
    idx = lambda i, j: i * (n + 1) + j + 1
    conn = np.array([[idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
                     for i in range(n) for j in range(n)])
    dof = np.arange(1, 6 * xyz.shape[0] + 1).reshape(-1, 6)
    q = np.array([0, 0, -2.5, 0, 0, 0.0])
    F = O.distribloads(xyz, conn, dof, order, 2, q, dof.size)
    X = xyz[conn - 1]
    A = np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 3] - X[:, 0]), axis=1)
    ref = np.zeros(xyz.shape[0])
    for e in range(conn.shape[0]):
        ref[conn[e] - 1] += -2.5 * A[e] / 4
    assert np.abs(F[dof[:, 2] - 1] - ref).max() <= 1e-14 * np.abs(ref).max()
    assert np.all(F[dof[:, [0, 1, 3, 4, 5]] - 1] == 0.0)


@pytest.mark.parametrize("rule", [3, 6])
def test_linear_field_per_point_is_integrated_exactly(rule):
    # f_z = x at the points: the consistent load of a linear field on a
    # triangle is A/12 (2 x_a + x_b + x_c), exact for rules of degree >= 2
    xyz, conn, dof, _ = PB.jittered_plate(4, False, jitter=0.2, wavy=0.0, seed=5, clamp_x0=False)
    pts = O.integration_points(xyz, conn, rule)
    f = np.zeros((pts.shape[0], 6))
    f[:, 2] = pts[:, 0]
    F = O.distribloads(xyz, conn, dof, rule, 3, f, int(dof.max()))
    A = _areas(xyz, conn)
    ref = np.zeros(xyz.shape[0])
    for e in range(conn.shape[0]):
        x = xyz[conn[e] - 1, 0]
        for a in range(3):
            ref[conn[e, a] - 1] += A[e] / 12 * (x.sum() + x[a])
    assert np.abs(F[dof[:, 2] - 1] - ref).max() <= 1e-13 * np.abs(ref).max()


def test_points_and_per_element_force():
    xyz, conn, dof, _ = PB.jittered_plate(3, True, jitter=0.1, wavy=0.02, seed=1, clamp_x0=False)
    pts = O.integration_points(xyz, conn, 2)
    assert pts.shape == (4 * conn.shape[0], 9)
    # points are inside the element's bounding box; tangents of a flat-ish quad
    X = xyz[conn[0] - 1]
    assert np.all(pts[:4, :3] >= X.min(axis=0) - 1e-12) and np.all(pts[:4, :3] <= X.max(axis=0) + 1e-12)
    # one force per element equals the same force repeated at every point
    rng = np.random.default_rng(4)
    fe = rng.normal(size=(conn.shape[0], 6))
    F1 = O.distribloads(xyz, conn, dof, 2, 3, fe, int(dof.max()))
    F2 = O.distribloads(xyz, conn, dof, 2, 3, np.repeat(fe, 4, axis=0), int(dof.max()))
    assert np.array_equal(F1, F2)


def test_scordelis_lo_load_matches_the_pinned_one():
    # PB.surface_load is the load under which the GPU stiffness reproduces the
    # reference's Scordelis-Lo deflection (test_gpu_parity)
    for quads, rule in ((False, 3), (True, 2)):
        d = PB.scordelis_lo(quads, 8)
        F = O.distribloads(d["xyz"], d["conn"], d["dofnums"], rule, 3, [0, 0, -90.0, 0, 0, 0],
                           int(d["dofnums"].max()))
        assert np.abs(F - d["F"]).max() <= 1e-13 * np.abs(d["F"]).max()


def test_free_block_and_bad_arguments():
    xyz, conn, dof, nfree = PB.jittered_plate(4, False, seed=3)
    q = [0, 0, -1.0, 0, 0, 0]
    Fa = O.distribloads(xyz, conn, dof, 1, 3, q, int(dof.max()))
    Ff = O.distribloads(xyz, conn, dof, 1, 3, q, nfree)
    assert np.array_equal(Fa[:nfree], Ff)
    with pytest.raises(RuntimeError):
        O.distribloads(xyz, conn, dof, 4, 3, q, nfree)
    with pytest.raises(RuntimeError):
        O.distribloads(xyz, conn, dof, 1, 1, q, nfree)
    with pytest.raises(RuntimeError):
        O.distribloads(xyz, conn, dof, 1, 3, np.zeros((5, 6)), nfree)

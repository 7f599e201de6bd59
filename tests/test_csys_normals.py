"""Nodal normals from a built-in material csys (associategeometry! with a
FEMM mcsys other than the isoparametric one: src/FEMMShellT3FFModule.jl:
570-616, src/FEMMShellQ4RSModule.jl:472-525, with the csys kinds the reference
examples define as closures).  The oracle is checked here on closed-form
geometry (CPU); tests/test_gpu_csys_normals.py compares the GPU with it."""
import numpy as np
import pytest

from oracle import oracle as O

E, NU = 2.0e11, 0.3
DPS = E / (1 - NU ** 2) * np.array([[1, NU, 0], [NU, 1, 0], [0, 0, (1 - NU) / 2]])
MAT = dict(Dps=DPS, Dt=E / 2 / (1 + NU) * np.eye(2), rho=7850.0)


def cylinder_panel(quads, nc=6, nl=5, R=2.0, L=3.0, half=np.radians(40)):
    """Panel of the cylinder of radius R around the y axis (the cylindrical!
    of the reference examples): nodes (R sin t, y, R cos t)."""
    th = np.linspace(-half, half, nc + 1)
    ys = np.linspace(0.0, L, nl + 1)
    T, Y = np.meshgrid(th, ys, indexing="ij")
    xyz = np.c_[R * np.sin(T.ravel()), Y.ravel(), R * np.cos(T.ravel())]
    idx = lambda i, j: i * (nl + 1) + j + 1
    conn = []
    for i in range(nc):
        for j in range(nl):
            q = [idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
            conn += [q] if quads else [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
    return xyz, np.array(conn)


def flat_plate(quads, n=4):
    xs, ys = np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    xyz = np.c_[xs.ravel(), ys.ravel(), np.zeros(xs.size)]
    idx = lambda i, j: i * (n + 1) + j + 1
    conn = []
    for i in range(n):
        for j in range(n):
            q = [idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
            conn += [q] if quads else [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
    return xyz, np.array(conn)


def _problem(xyz, conn):
    et = O.Q4RS if conn.shape[1] == 4 else O.T3FF
    return O.Problem(et, xyz, conn, None, thickness=0.01, material=MAT)


@pytest.mark.parametrize("quads", [False, True])
def test_cylindrical_csys_gives_radial_normals(quads):
    xyz, conn = cylinder_panel(quads)
    P = _problem(xyz, conn)
    nrm, val = P.compute_normals(30.0, O.CSYS_CYLINDRICAL, [0, 0, 0, 0, 1, 0])
    r = xyz * [1, 0, 1]
    ref = r / np.linalg.norm(r, axis=1)[:, None]
    assert np.abs(nrm - ref).max() <= 1e-15
    assert np.all(val == 1)


@pytest.mark.parametrize("quads", [False, True])
def test_spherical_csys_gives_radial_normals(quads):
    xyz, conn = cylinder_panel(quads)
    c = np.array([0.3, 1.0, -0.5])
    P = _problem(xyz, conn)
    nrm, _ = P.compute_normals(30.0, O.CSYS_SPHERICAL, c)
    ref = (xyz - c) / np.linalg.norm(xyz - c, axis=1)[:, None]
    assert np.abs(nrm - ref).max() <= 1e-15


def test_validity_test_differs_between_t3_and_q4():
    # a cartesian csys whose third axis lies in the plane of a flat plate:
    # T3 compares the nodal normal with the element frame normal (all nodes
    # invalid), Q4 with the csys normal itself (all valid)
    cs = np.column_stack([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])  # third column = x
    for quads, expect in ((False, 0), (True, 1)):
        xyz, conn = flat_plate(quads)
        P = _problem(xyz, conn)
        nrm, val = P.compute_normals(30.0, O.CSYS_CARTESIAN, cs)
        assert np.allclose(nrm, [1.0, 0.0, 0.0], atol=1e-15)
        assert np.all(val == expect)

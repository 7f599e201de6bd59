"""Stress resultants at the integration points (inspectintegpoints of
FEMMShellT3FF, src/FEMMShellT3FFModule.jl:850-962, and FEMMShellQ4RS,
src/FEMMShellQ4RSModule.jl:1061-1170).  CPU only.

The reference's tests call inspectintegpoints only inside examples, with no
recorded values, so the oracle's restatement is pinned here by closed-form
states of a flat plate: a uniform stretch gives n = t Dps eps, a uniform
curvature gives m = t^3/12 Dps kappa, a uniform transverse shear gives
q = t stab (5/6) G gamma.  The library's point math, built for the host
(tests/hostcheck), is then compared with the oracle on the curved
Scordelis-Lo roof with random displacements and output frames."""
import numpy as np
import pytest

from oracle import oracle as O
from flexshell import _abi
from hostcheck import hostmath as HC
import problems as PB
from test_hostcheck import _homog

E, NU, T = 200e9, 0.3, 0.01
DPS = E / (1 - NU ** 2) * np.array([[1, NU, 0], [NU, 1, 0], [0, 0, (1 - NU) / 2]])
G = E / 2 / (1 + NU)


def _plate(quads, jitter):
    xyz, conn, dof, _ = PB.jittered_plate(6, quads, jitter=jitter, wavy=0.0, seed=3)
    P = O.Problem(O.Q4RS if quads else O.T3FF, xyz, conn, dof, thickness=T,
                  material=dict(Dps=DPS, Dt=G * np.eye(2), rho=7850.0))
    P.compute_normals()
    return xyz, P


@pytest.mark.parametrize("quads", [False, True])
def test_oracle_membrane_and_bending_closed_form(quads):
    xyz, P = _plate(quads, 0.2)
    x = xyz[:, 0]
    u = np.zeros((xyz.shape[0], 6))
    eps = 1e-3
    u[:, 0] = eps * x                          # u = eps x: n_xx = t D11 eps, n_yy = t D21 eps
    r = P.resultants(u, O.RES_MEMBRANE, np.eye(3))
    ref = T * DPS[:, 0] * eps
    assert np.abs(r - ref).max() <= 1e-10 * np.abs(ref).max()
    u[:] = 0.0
    kap = 1e-2
    u[:, 4] = kap * x                          # rotation about y = kappa x: kappa_xx = kappa
    u[:, 2] = kap * x ** 2 / 2
    r = P.resultants(u, O.RES_MOMENT, np.eye(3))
    ref = T ** 3 / 12 * DPS[:, 0] * kap
    assert np.abs(r - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("quads", [False, True])
def test_oracle_transverse_shear_closed_form(quads):
    # T3 (DSG, averaged over the node orderings) reproduces a constant shear on
    # a distorted mesh; the Q4 MITC rows do so on a regular mesh
    xyz, P = _plate(quads, 0.0 if quads else 0.2)
    u = np.zeros((xyz.shape[0], 6))
    gam = 1e-3
    u[:, 2] = gam * xyz[:, 0]                  # w = gamma x, no rotation: gamma_xz = gamma
    r = P.resultants(u, O.RES_SHEAR, np.eye(3))
    X = xyz[P.conn - 1]
    if quads:
        h2 = np.max([np.sum((X[:, k] - X[:, 0]) ** 2, axis=1) for k in (1, 2, 3)], axis=0)
        stab = np.repeat(T ** 2 / (T ** 2 + 0.1 * h2), 4)
    else:
        Ae = 0.5 * np.abs(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0])[:, 2])
        stab = T ** 2 / (T ** 2 + (5 / 12 / 1.5) * 2 * Ae)
    ref = T * stab * (5 / 6) * G * gam
    assert np.abs(r[:, 0] - ref).max() <= 1e-10 * ref.max()
    assert np.abs(r[:, 1:]).max() <= 1e-10 * ref.max()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("quantity", [_abi.FS_RES_MOMENT, _abi.FS_RES_SHEAR, _abi.FS_RES_MEMBRANE])
@pytest.mark.parametrize("frame", ["element", "one", "per_point"])
def test_host_point_math_matches_oracle(quads, quantity, frame):
    et, d, P, prm = _homog(quads, n=6)
    rng = np.random.default_rng(7)
    u = rng.normal(size=(d["xyz"].shape[0], 6)) * 1e-3
    npt = P.nelem * (4 if quads else 1)
    cs = {"element": None, "one": np.linalg.qr(rng.normal(size=(3, 3)))[0],
          "per_point": np.linalg.qr(rng.normal(size=(npt, 3, 3)))[0]}[frame]
    ro = P.resultants(u, quantity, cs)
    rh = HC.resultants(et, d["xyz"], d["conn"], P.normals, P.valid, d["thickness"], prm, u, quantity, cs)
    assert np.abs(rh - ro).max() <= 1e-13 * np.abs(ro).max()
    if quantity == _abi.FS_RES_SHEAR:
        assert np.all(ro[:, 2] == 0.0)

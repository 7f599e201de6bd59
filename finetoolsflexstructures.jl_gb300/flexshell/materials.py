"""Material stiffness helpers (host side, computed once per call).

``tangentmoduli`` restates the FinEtoolsDeforLinear 3.0.6 3D stiffness of
``MatDeforElastIso`` and ``MatDeforElastOrtho`` (ordering xx, yy, zz, xy,
xz, yz).  ``shell_material_stiffness`` is the plane-stress reduction of the
reference, src/FEMMShellT3FFModule.jl:323-342 (same in the Q4RS module
:266-285 and in ``Ply``, src/CompositeLayupModule.jl:78-96).
"""
import numpy as np


class MatDeforElastIso:
    def __init__(self, E, nu, rho=0.0):
        self.E, self.nu, self.rho = float(E), float(nu), float(rho)

    def tangentmoduli(self):
        E, nu = self.E, self.nu
        lam = E * nu / (1 + nu) / (1 - 2 * nu)
        mu = E / 2.0 / (1 + nu)
        m1 = np.array([1.0, 1.0, 1.0, 0.0, 0.0, 0.0])
        mI = np.diag([1.0, 1.0, 1.0, 0.5, 0.5, 0.5])
        return lam * np.outer(m1, m1) + 2.0 * mu * mI

    def massdensity(self):
        return self.rho


class MatDeforElastOrtho:
    def __init__(self, E1, E2, E3, nu12, nu13, nu23, G12, G13, G23, rho=0.0):
        self.p = (float(E1), float(E2), float(E3), float(nu12), float(nu13), float(nu23),
                  float(G12), float(G13), float(G23))
        self.rho = float(rho)

    def tangentmoduli(self):
        E1, E2, E3, nu12, nu13, nu23, G12, G13, G23 = self.p
        C = np.array([
            [1.0 / E1, -nu12 / E1, -nu13 / E1, 0, 0, 0],
            [-nu12 / E1, 1.0 / E2, -nu23 / E2, 0, 0, 0],
            [-nu13 / E1, -nu23 / E2, 1.0 / E3, 0, 0, 0],
            [0, 0, 0, 1 / G12, 0, 0],
            [0, 0, 0, 0, 1 / G13, 0],
            [0, 0, 0, 0, 0, 1 / G23],
        ])
        return np.linalg.inv(C)

    def massdensity(self):
        return self.rho


def lamina_material(*args):
    """CompositeLayupModule.lamina_material, src/CompositeLayupModule.jl:105-167:
    (E1,E2,nu12,G12,G13,G23), (rho,E1,E2,nu12,G12,G13,G23), (E,nu), (rho,E,nu)."""
    if len(args) == 6:
        E1, E2, nu12, G12, G13, G23 = args
        return MatDeforElastOrtho(E1, E2, E2, nu12, nu12, 0.0, G12, G13, G23, 0.0)
    if len(args) == 7:
        rho, E1, E2, nu12, G12, G13, G23 = args
        return MatDeforElastOrtho(E1, E2, E2, nu12, nu12, 0.0, G12, G13, G23, rho)
    if len(args) == 2:
        return MatDeforElastIso(args[0], args[1], 0.0)
    if len(args) == 3:
        return MatDeforElastIso(args[1], args[2], args[0])
    raise TypeError("unsupported lamina_material arguments")


def shell_material_stiffness(material):
    """(Dps 3x3, Dt 2x2) from the 3D stiffness: plane-stress reduction and the
    transverse shear diagonal (the 5/6 factor is applied by the element)."""
    D = material.tangentmoduli()
    Dps = np.zeros((3, 3))
    Dps[0:2, 0:2] = D[0:2, 0:2] - np.outer(D[0:2, 2], D[2, 0:2]) / D[2, 2]
    ix = [0, 1, 3]
    for i in range(3):
        Dps[2, i] = Dps[i, 2] = D[3, ix[i]]
    Dt = np.zeros((2, 2))
    Dt[0, 0] = D[4, 4]
    Dt[1, 1] = D[5, 5]
    return Dps, Dt

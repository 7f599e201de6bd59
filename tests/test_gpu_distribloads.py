"""GPU parity of the distributed surface loads (fs_distribloads,
fs_integration_points: FinEtools distribloads on the shell element sets, as
test/test_shell_statics.jl:84-86 and plate_expl_examples.jl:196-199 call it)
against the oracle, through the Python mirror and the C ABI.  Tolerance 1e-12
relative (max-abs difference over max-abs value)."""
import numpy as np
import pytest

import flexshell as F
from flexshell import _abi
from flexshell._lib import FlexShellError, ptr
from oracle import oracle as O
import problems as PB

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _setup(quads, n=8):
    d = PB.scordelis_lo(quads, n)
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    return d, F.NodalField(d["xyz"]), dchi


@pytest.mark.parametrize("quads", [False, True])
def test_uniform_and_per_point_loads_match_oracle(quads):
    d, geom0, dchi = _setup(quads)
    rules = (F.GaussRule(2, 1), F.GaussRule(2, 2), F.GaussRule(2, 3)) if quads else \
        (F.TriRule(1), F.TriRule(3), F.TriRule(6))
    q = np.array([0.5, -0.25, -90.0, 0.01, -0.02, 0.03])
    n = dchi.nalldofs()
    for rule in rules:
        lfemm = F.FEMMBase(F.IntegDomain(d["conn"], rule))
        for m in (2, 3):
            Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(q), m)
            Fo = O.distribloads(d["xyz"], d["conn"], d["dofnums"], rule.code, m, q, n)
            assert Fg.shape == (n,) and _rel(Fg, Fo) <= 1e-12
        # integration points, then a location-dependent callable (the example's
        # computetrac!: a pressure patch around a point)
        pts = lfemm.integration_points(geom0)
        po = O.integration_points(d["xyz"], d["conn"], rule.code)
        assert np.abs(pts - po).max() <= 1e-12 * np.abs(po).max()
        centre = d["xyz"][d["probe"]]
        calls = []

        def computetrac(forceout, XYZ, tangents, feid, qpid):
            calls.append((feid, qpid))
            assert tangents.shape == (3, 2)
            forceout[:] = 0.0
            if np.linalg.norm(XYZ.ravel() - centre) < 10.0:
                forceout[2] = -1000.0
            return forceout

        fi = F.ForceIntensity(float, 6, computetrac)
        Fg = F.distribloads(lfemm, F.SysvecAssemblerFBlock(dchi.nfreedofs), geom0, dchi, fi, 2)
        fpts = np.zeros((po.shape[0], 6))
        fpts[np.linalg.norm(po[:, :3] - centre, axis=1) < 10.0, 2] = -1000.0
        Fo = O.distribloads(d["xyz"], d["conn"], d["dofnums"], rule.code, 2, fpts, dchi.nfreedofs)
        assert Fg.shape == (dchi.nfreedofs,) and _rel(Fg, Fo) <= 1e-12
        assert calls[0] == (1, 1) and len(calls) == po.shape[0]
        lfemm.close()


def test_scordelis_lo_load_solves_to_the_reference_deflection():
    # the load from the GPU reproduces the pinned one; the solve against the
    # reference's deflection is test_gpu_parity's
    for quads, rule in ((False, F.TriRule(3)), (True, F.GaussRule(2, 2))):
        d, geom0, dchi = _setup(quads)
        lfemm = F.FEMMBase(F.IntegDomain(d["conn"], rule))
        Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity([0, 0, -90.0, 0, 0, 0]), 3)
        assert _rel(Fg, d["F"]) <= 1e-12
        lfemm.close()


def test_per_element_force_and_errors():
    d, geom0, dchi = _setup(False, 4)
    lfemm = F.FEMMBase(F.IntegDomain(d["conn"], F.TriRule(3)))
    lfemm._sync(geom0, dchi)
    ctx = lfemm.ctx
    ne = d["conn"].shape[0]
    fe = np.random.default_rng(2).normal(size=(ne, 6))
    n = dchi.nalldofs()
    out = np.zeros(n)
    ctx.call("fs_distribloads", 3, 3, ptr(fe), ne, n, ptr(out))
    assert _rel(out, O.distribloads(d["xyz"], d["conn"], d["dofnums"], 3, 3, fe, n)) <= 1e-12
    for rule, m, nf in ((4, 3, 1), (3, 1, 1), (3, 3, 5)):
        with pytest.raises(FlexShellError) as ei:
            ctx.call("fs_distribloads", rule, m, ptr(fe), nf, n, ptr(out))
        assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    lfemm.close()

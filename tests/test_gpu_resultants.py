"""GPU parity of the integration-point resultants (fs_resultants, the
inspectintegpoints of FEMMShellT3FF and FEMMShellQ4RS) against the oracle,
through the C ABI and the Python mirror.  Tolerance 1e-12 relative (max-abs
difference over max-abs value) with given output frames.  With the default
frame (the element frame: the shells' mcsys updater is _e_g!) the output
angle comes from Layup2ElementAngle of a frame and itself, whose
n = sqrt(1 - m^2) turns a last-bit difference of m = 1 into about 1e-8 (the
reference carries the same noise), so that case is held to 1e-7."""
import ctypes

import numpy as np
import pytest

import flexshell as F
from flexshell import _abi
from flexshell._lib import FlexShellError, ptr
from oracle import oracle as O
import problems as PB
from test_gpu_parity import homog_pair

pytestmark = pytest.mark.gpu

QUANTS = [("bending", _abi.FS_RES_MOMENT), ("shear", _abi.FS_RES_SHEAR), ("membrane", _abi.FS_RES_MEMBRANE)]


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("quantity", QUANTS)
def test_resultants_match_oracle(quads, quantity):
    name, q = quantity
    d = PB.scordelis_lo(quads, 8)
    P, femm, geom0, _ = homog_pair(d, quads)
    rng = np.random.default_rng(11)
    u = rng.normal(size=(d["xyz"].shape[0], 6)) * 1e-3
    npt = P.nelem * (4 if quads else 1)
    one = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    per = np.linalg.qr(rng.normal(size=(npt, 3, 3)))[0]
    for cs, tol in ((one, 1e-12), (per, 1e-12), (None, 1e-7)):
        g = femm.resultants(geom0, u, name, cs)
        o = P.resultants(u, q, cs)
        assert g.shape == (npt, 3)
        assert _rel(g, o) <= tol
    # a callable frame is evaluated per point like updatecsmat!
    calls = []

    def ocsys(XYZ, tangents, feid, qpid):
        calls.append((feid, qpid))
        return per[len(calls) - 1]

    g = femm.resultants(geom0, u, name, ocsys)
    assert _rel(g, P.resultants(u, q, per)) <= 1e-12
    assert calls[0] == (1, 1 if quads else 0) and len(calls) == npt
    femm.close()


def test_inspectintegpoints_walks_felist():
    d = PB.scordelis_lo(True, 4)
    P, femm, geom0, _ = homog_pair(d, True)
    u = np.random.default_rng(3).normal(size=(d["xyz"].shape[0], 6)) * 1e-3
    felist = [5, 2, 9]

    def inspector(idat, i, conn, ecoords, out, loc):
        idat.append((i, out.copy(), loc.copy()))
        return idat

    idat = femm.inspectintegpoints(geom0, u, felist, inspector, [], "membrane")
    assert [x[0] for x in idat] == [5] * 4 + [2] * 4 + [9] * 4
    o = P.resultants(u, O.RES_MEMBRANE, None)
    for k, (i, out, loc) in enumerate(idat):
        assert np.abs(out - o[4 * (i - 1) + k % 4]).max() <= 1e-7 * np.abs(o).max()
        assert loc.shape == (1, 3)
    # the centroid-like Gauss points lie inside the element's bounding box
    X = d["xyz"][d["conn"][4] - 1]
    assert np.all(idat[0][2] >= X.min(axis=0) - 1e-12) and np.all(idat[0][2] <= X.max(axis=0) + 1e-12)
    femm.close()


def test_resultants_errors():
    d = PB.scordelis_lo(False, 4)
    P, femm, geom0, _ = homog_pair(d, False)
    ctx = femm.ctx
    u = np.zeros((d["xyz"].shape[0], 6))
    out = np.zeros((P.nelem, 3))
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_resultants", 7, ptr(u), None, 0, ptr(out))
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    cs = np.eye(3)
    with pytest.raises(FlexShellError) as ei:
        ctx.call("fs_resultants", _abi.FS_RES_MOMENT, ptr(u), ptr(cs), 2, ptr(out))
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    femm.close()
    # normals are required (associategeometry!)
    femm = F.FEMMShellT3FF(d["conn"], d["thickness"], femm.material, stab_fun=d["stab_c"])
    femm._upload_mesh(geom0)
    with pytest.raises(FlexShellError) as ei:
        femm.ctx.call("fs_resultants", _abi.FS_RES_MOMENT, ptr(u), None, 0, ptr(out))
    assert ei.value.code == _abi.FS_ERR_STATE
    femm.close()
    # layered shells: not this entry point
    xyz, conn, dof, nfree, plies = PB.c4_plate(4)
    fc = F.FEMMShellQ4RSComp(conn, F.laminate(plies))
    g0 = F.NodalField(xyz)
    fc.associategeometry(g0)
    uu = np.zeros((xyz.shape[0], 6))
    oo = np.zeros((4 * conn.shape[0], 3))
    with pytest.raises(FlexShellError) as ei:
        fc.ctx.call("fs_resultants", _abi.FS_RES_MOMENT, ptr(uu), None, 0, ptr(oo))
    assert ei.value.code == _abi.FS_ERR_UNSUPPORTED
    fc.close()

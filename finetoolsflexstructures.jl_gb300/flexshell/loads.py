"""Distributed loads on the shell meshes, the FinEtools 8.2.5 calls the
reference makes around its shell FEMMs:

    lfemm = FEMMBase(IntegDomain(fes, TriRule(3)))                 # or GaussRule(2, 2)
    fi = ForceIntensity([0, 0, -q, 0, 0, 0])                       # or a callable
    F = distribloads(lfemm, geom0, dchi, fi, 3)                    # test/test_shell_statics.jl:84-86
    Fmag = distribloads(lfemm, vassem, geom0, dchi, fi, 2)         # plate_expl_examples.jl:196-199
    bfes = mesh.meshboundary(fes)                                  # edge loads on boundary curves:
    lfemm = FEMMBase(IntegDomain(bfes[l1], GaussRule(1, 2)))       # test/test_shell_statics.jl:212-215

The element loop and the per-node sums run in libflexshell.so
(fs_distribloads); a callable ForceIntensity is evaluated on the host at the
integration points the library returns (fs_integration_points), as the
reference evaluates its closure point by point.
"""
import numpy as np

from ._lib import Context, ptr
from . import _abi


class TriRule:
    """TriRule(npts): 1, 3 or 6 points on the triangle."""

    def __init__(self, npts=1):
        if npts not in (1, 3, 6):
            raise ValueError("TriRule: npts 1, 3 or 6")
        self.npts = npts
        self.code = npts


class GaussRule:
    """GaussRule(2, order): order x order points on the quadrilateral;
    GaussRule(1, order): order points on the two-node line element."""

    def __init__(self, dim, order):
        if dim not in (1, 2) or order not in (1, 2, 3):
            raise ValueError("GaussRule: dim 1 or 2, order 1, 2 or 3")
        self.dim = dim
        self.npts = order ** dim
        self.code = order


class IntegDomain:
    """IntegDomain(fes, rule): the element set (connectivity, nelem x 2
    line elements, nelem x 3 triangles or nelem x 4 quadrilaterals, 1-based)
    and its integration rule."""

    def __init__(self, conn, rule):
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        if self.conn.ndim != 2 or self.conn.shape[1] not in (2, 3, 4):
            raise ValueError("IntegDomain: lines (nelem x 2), triangles (nelem x 3) or quadrilaterals (nelem x 4)")
        nen = self.conn.shape[1]
        ok = isinstance(rule, TriRule) if nen == 3 else (isinstance(rule, GaussRule) and rule.dim == nen // 2)
        if not ok:
            raise ValueError("IntegDomain: GaussRule(1, order) for lines, TriRule for triangles, "
                             "GaussRule(2, order) for quadrilaterals")
        self.rule = rule


class ForceIntensity:
    """ForceIntensity(vector) or ForceIntensity(callable): the callable is
    computetrac!(forceout, XYZ, tangents, feid, qpid) of the reference (fills
    the six components of forceout; XYZ 1 x 3, tangents 3 x 2, feid the
    1-based element, qpid the 1-based point)."""

    def __init__(self, *args):
        # ForceIntensity(vector), ForceIntensity(fun) or ForceIntensity(Float64, 6, fun)
        f = args[-1]
        ncomp = int(args[1]) if len(args) == 3 else 6
        if ncomp != 6:
            raise ValueError("ForceIntensity: six components (one per nodal dof)")
        if callable(f):
            self.fun, self.value = f, None
        else:
            v = np.asarray(f, dtype=np.float64).ravel()
            if v.shape[0] != 6:
                raise ValueError("ForceIntensity: six components (one per nodal dof)")
            self.fun, self.value = None, v
        self.ncomp = ncomp


class SysvecAssembler:
    """Vector of all the dofs (nalldofs)."""
    nrows = None


class SysvecAssemblerFBlock:
    """Free block: dofs above nfreedofs are left out."""

    def __init__(self, nfree):
        self.nrows = int(nfree)


class FEMMBase:
    """FEMMBase(integdomain): the load integrals of an element set, on the GPU."""

    def __init__(self, integdomain, device=0):
        self.integdomain = integdomain
        self.ctx = Context(device)
        self._key = None

    def _upload(self, geom):
        xyz = np.asfortranarray(geom.values, dtype=np.float64)
        key = (xyz.shape, xyz.tobytes())
        if key != self._key:
            conn = self.integdomain.conn
            # a two-node set goes in as the library's two-node (beam) mesh type
            et = {2: _abi.FS_COROTBEAM, 3: _abi.FS_T3FF, 4: _abi.FS_Q4RS}[conn.shape[1]]
            self.ctx.call("fs_mesh_set", et, xyz.shape[0], ptr(xyz), conn.shape[0], ptr(conn), None, None)
            self._key = key

    def _sync(self, geom, dchi):
        self._upload(geom)
        d = np.asfortranarray(dchi.dofnums, dtype=np.int64)
        self.ctx.call("fs_dofs_set", ptr(d))

    def integration_points(self, geom):
        """(npoints, 9): location, x_xi, x_eta of every point, element order
        (x_eta zero on line elements)."""
        self._upload(geom)
        rule = self.integdomain.rule
        out = np.zeros((self.integdomain.conn.shape[0] * rule.npts, 9))
        self.ctx.call("fs_integration_points", rule.code, ptr(out))
        return out

    def close(self):
        self.ctx.close()


def distribloads(femm, *args):
    """distribloads(femm, [assembler,] geom, P, fi, m): the load vector of
    the force intensity fi over the element set (m = 2 or 3 on surfaces, 1, 2
    or 3 on lines; the elements' other dimension is 1).  Returns nalldofs(P)
    entries, or nfreedofs with SysvecAssemblerFBlock."""
    if len(args) == 4:
        assembler, (geom, P, fi, m) = SysvecAssembler(), args
    elif len(args) == 5:
        assembler, geom, P, fi, m = args
    else:
        raise TypeError("distribloads(femm, [assembler,] geom, P, fi, m)")
    femm._sync(geom, P)
    rule = femm.integdomain.rule
    conn = femm.integdomain.conn
    if fi.fun is None:
        force = fi.value
    else:
        pts = femm.integration_points(geom)
        force = np.zeros((pts.shape[0], 6))
        k = 0
        for e in range(conn.shape[0]):
            for j in range(rule.npts):
                out = np.zeros(6)
                tang = (pts[k, 3:6].reshape(3, 1) if conn.shape[1] == 2
                        else np.column_stack([pts[k, 3:6], pts[k, 6:9]]))
                r = fi.fun(out, pts[k, 0:3].reshape(1, 3), tang, e + 1, j + 1)
                force[k] = out if r is None else np.asarray(r, dtype=np.float64).ravel()[:6]
                k += 1
    force = np.ascontiguousarray(force, dtype=np.float64).reshape(-1, 6)
    n = P.nalldofs() if assembler.nrows is None else assembler.nrows
    F = np.zeros(n)
    femm.ctx.call("fs_distribloads", rule.code, int(m), ptr(force), force.shape[0], n, ptr(F))
    return F

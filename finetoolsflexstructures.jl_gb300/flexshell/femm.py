"""Host mirror of the reference FEMM interface for the shell hot path.

The classes keep the reference names and call pattern
(FinEtoolsFlexStructures.jl 3.6.4):

    femm = FEMMShellT3FF.make(fes, thickness, material, stab_fun)   # src/FEMMShellT3FFModule.jl:241-268
    femm.associategeometry(geom0)                                    # :570-616
    K = femm.stiffness(assembler, geom0, u1, Rfield1, dchi)          # :635-736
    M = femm.mass(assembler, geom0, dchi)                            # :757-811

and the same for FEMMShellQ4RS (src/FEMMShellQ4RSModule.jl),
FEMMShellT3FFComp and FEMMShellQ4RSComp (layup groups).  Matrices are
returned as scipy.sparse CSC (SparseMatrixCSC) or CSR
(SysmatAssemblerSparseCSRSymm) matrices.  All computation runs in
libflexshell.so on the GPU; `u1` and `Rfield1` are accepted and ignored as in
the reference shells.
"""
import numpy as np

from . import _abi, mesh as _mesh
from ._lib import Context, FlexShellError, InputCache, ptr

FS_FP64, FS_MIXED, FS_MIXED_COMP = _abi.FS_FP64, _abi.FS_MIXED, _abi.FS_MIXED_COMP


# ---------------------------------------------------------------------------
# fields and assemblers (FinEtools)
# ---------------------------------------------------------------------------
class NodalField:
    """FinEtools NodalField: values (nents x ndofn), fixed flags, dof numbers."""

    def __init__(self, values):
        self.values = np.array(values, dtype=np.float64, order="F")
        if self.values.ndim == 1:
            self.values = self.values[:, None]
        self.is_fixed = np.zeros(self.values.shape, dtype=bool)
        self.dofnums = np.zeros(self.values.shape, dtype=np.int64, order="F")
        self.nfreedofs = 0

    def setebc(self, nodes, comp):
        """Fix component `comp` (1-based) of the 1-based `nodes`."""
        self.is_fixed[np.asarray(nodes, dtype=np.int64) - 1, comp - 1] = True

    def numberdofs(self):
        d, nf = _mesh.numberdofs(self.is_fixed)
        self.dofnums = np.asfortranarray(d)
        self.nfreedofs = nf
        return self

    def nalldofs(self):
        return int(self.values.size)


class _Assembler:
    mode = _abi.FS_ASM_SPARSE
    csr = False
    nrows = None  # None: nalldofs(dchi)


class SysmatAssemblerSparseSymm(_Assembler):
    mode = _abi.FS_ASM_SPARSE_SYMM


class SysmatAssemblerSparse(_Assembler):
    mode = _abi.FS_ASM_SPARSE


class SysmatAssemblerSparseCSRSymm(_Assembler):
    """src/AssemblyModule.jl:20-53: SysmatAssemblerSparse result converted to CSR."""
    mode = _abi.FS_ASM_SPARSE
    csr = True


class SysmatAssemblerSparseDiag(_Assembler):
    mode = _abi.FS_ASM_DIAG


class SysmatAssemblerFFBlock(_Assembler):
    """Free-free block: dofs above nfreedofs are left out."""

    def __init__(self, a=None, nfree=None, ncfree=None):
        if nfree is None and isinstance(a, (int, np.integer)):
            a, nfree = None, int(a)
        inner = a if a is not None else SysmatAssemblerSparse()
        self.mode = inner.mode
        self.csr = inner.csr
        self.nrows = int(nfree)


# ---------------------------------------------------------------------------
# stab_fun family
# ---------------------------------------------------------------------------
def stab_coefficient(stab_fun, default):
    """The coefficient c of stab_fun(t, h) = t^2/(t^2 + c h^2).  Closures
    outside this family are rejected (ArgumentError in the Julia shim)."""
    if stab_fun is None:
        return default
    if isinstance(stab_fun, (int, float)):
        return float(stab_fun)
    f1 = float(stab_fun(1.0, 1.0))
    c = 1.0 / f1 - 1.0
    for t, h in ((0.3, 2.0), (0.01, 0.05)):
        want = t * t / (t * t + c * h * h)
        got = float(stab_fun(t, h))
        if abs(got - want) > 1e-12 * max(abs(want), 1e-300):
            raise ValueError("stab_fun is not of the form t^2/(t^2 + c h^2)")
    return c


# ---------------------------------------------------------------------------
# FEMMs
# ---------------------------------------------------------------------------
class CSysCartesian:
    """A fixed material csys (the reference examples' cartesian!): its third
    column is every node's normal."""
    kind = _abi.FS_CSYS_CARTESIAN

    def __init__(self, csmat=np.eye(3)):
        self.params = np.asarray(csmat, dtype=np.float64).flatten(order="F")


class CSysCylindrical:
    """Radial normals from an axis (the reference examples' cylindrical!,
    there the y axis through the origin)."""
    kind = _abi.FS_CSYS_CYLINDRICAL

    def __init__(self, point=(0.0, 0.0, 0.0), axis=(0.0, 1.0, 0.0)):
        a = np.asarray(axis, dtype=np.float64)
        self.params = np.r_[np.asarray(point, dtype=np.float64), a / np.linalg.norm(a)]


class CSysSpherical:
    """Radial normals from a centre (the reference examples' spherical!)."""
    kind = _abi.FS_CSYS_SPHERICAL

    def __init__(self, center=(0.0, 0.0, 0.0)):
        self.params = np.asarray(center, dtype=np.float64)


class _FEMMShell:
    etype = None
    nen = None
    default_stab = None

    def __init__(self, conn, thickness, material=None, stab_fun=None, device=0, layup_groups=None, mcsys=None):
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        if self.conn.ndim != 2 or self.conn.shape[1] != self.nen:
            raise ValueError("connectivity must be nelem x %d" % self.nen)
        self.material = material
        self.thickness = thickness
        self.stab_c = stab_coefficient(stab_fun, self.default_stab)
        self.transv_shear_formulation = 0
        self.drilling_stiffness_scale = 1.0
        self.threshold_angle = 30.0
        self.layup_groups = layup_groups
        self.mcsys = mcsys  # None: isoparametric (the reference default); or a CSys* above
        self.ctx = Context(device)
        self._geom = InputCache()
        self._dofs = InputCache()
        self._associatedgeometry = False
        self._normals = None
        self._normal_valid = None

    # -- parameters -------------------------------------------------------
    def _params(self):
        from .materials import shell_material_stiffness
        if self.material is not None:
            Dps, Dt = shell_material_stiffness(self.material)
            rho = self.material.massdensity()
        else:
            Dps, Dt, rho = np.eye(3), np.eye(2), 0.0
        th = self.thickness
        scalar_t = float(th) if np.isscalar(th) else 0.0
        p = _abi.make_params(Dps, Dt, rho, scalar_t, stab_c=self.stab_c,
                             drilling_stiffness_scale=self.drilling_stiffness_scale,
                             threshold_angle=self.threshold_angle,
                             transv_shear_formulation=self.transv_shear_formulation)
        tharr = None if np.isscalar(th) or th is None else np.ascontiguousarray(th, dtype=np.float64)
        return p, tharr

    def _order(self):
        if not self.layup_groups:
            return None
        return np.ascontiguousarray(np.concatenate([np.asarray(g[1], dtype=np.int64)
                                                    for g in self.layup_groups]))

    def _upload_mesh(self, geom0):
        xyz = np.asfortranarray(geom0.values, dtype=np.float64)
        order = self._order()
        self.ctx.call("fs_mesh_set", self.etype, xyz.shape[0], ptr(xyz), self.conn.shape[0],
                      ptr(self.conn), ptr(order), None)
        p, tharr = self._params()
        self.ctx.call("fs_params_set", p, ptr(tharr))
        if self.layup_groups:
            groups = [g[0] for g in self.layup_groups]
            eg = np.zeros(self.conn.shape[0], dtype=np.int32)
            for k, g in enumerate(self.layup_groups):
                eg[np.asarray(g[1], dtype=np.int64) - 1] = k
            arr = (_abi.fs_layup_group * len(groups))(*groups)
            self.ctx.call("fs_layups_set", len(groups), arr, ptr(eg))
        self._geom.store(xyz)
        self._dofs.clear()

    def _sync_inputs(self, geom0, dchi):
        xyz = np.asfortranarray(geom0.values, dtype=np.float64)
        if self._geom.copy is not None and xyz.shape != self._geom.copy.shape:
            raise ValueError("geometry with %d nodes for a mesh of %d: call associategeometry with it first"
                             % (xyz.shape[0], self._geom.copy.shape[0]))
        if self._geom.stale(xyz):
            self.ctx.call("fs_geometry_set", ptr(xyz))
            self._geom.store(xyz)
        p, tharr = self._params()
        self.ctx.call("fs_params_set", p, ptr(tharr))
        if dchi is not None:
            d = np.asfortranarray(dchi.dofnums, dtype=np.int64)
            if d.shape != (geom0.values.shape[0], 6):
                raise ValueError("dchi must have 6 dofs per node")
            if self._dofs.stale(d):
                self.ctx.call("fs_dofs_set", ptr(d))
                self._dofs.store(d)

    # -- reference interface --------------------------------------------------
    def associategeometry(self, geom0):
        """associategeometry!(femm, geom0): nodal normals and validity."""
        self._upload_mesh(geom0)
        if self.mcsys is None:
            self.ctx.call("fs_normals_compute")
        else:
            prm = np.ascontiguousarray(self.mcsys.params, dtype=np.float64)
            self.ctx.call("fs_normals_compute_csys", self.mcsys.kind, ptr(prm))
        nn = geom0.values.shape[0]
        self._normals = np.zeros((nn, 3), order="F")
        self._normal_valid = np.zeros(nn, dtype=np.uint8)
        self.ctx.call("fs_normals_get", ptr(self._normals), ptr(self._normal_valid))
        self._associatedgeometry = True
        return self

    def set_normals(self, normals, valid):
        """Normals from a user coordinate system (the reference's `mcsys`)."""
        self._normals = np.asfortranarray(normals, dtype=np.float64)
        self._normal_valid = np.ascontiguousarray(valid, dtype=np.uint8)
        self.ctx.call("fs_normals_set", ptr(self._normals), ptr(self._normal_valid))
        self._associatedgeometry = True

    def _fetch(self, nrows, nnz, csr):
        import scipy.sparse as sp
        colptr = np.empty(nrows + 1, dtype=np.int64)
        rowval = np.empty(nnz, dtype=np.int64)
        nzval = np.empty(nnz, dtype=np.float64)
        self.ctx.call("fs_matrix_copy", ptr(colptr), ptr(rowval), ptr(nzval))
        if csr:
            return sp.csr_matrix((nzval, rowval - 1, colptr - 1), shape=(nrows, nrows))
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(nrows, nrows))

    def stiffness(self, assembler, geom0, u1=None, Rfield1=None, dchi=None, precision=FS_FP64):
        """stiffness(femm, assembler, geom0, u1, Rfield1, dchi) -> K."""
        if not isinstance(assembler, _Assembler):
            # stiffness(femm, geom0, u1, Rfield1, dchi): default assembler
            assembler, geom0, u1, Rfield1, dchi = SysmatAssemblerSparseSymm(), assembler, geom0, u1, Rfield1
        if not self._associatedgeometry:
            raise AssertionError("self._associatedgeometry == true")
        self._sync_inputs(geom0, dchi)
        nrows = assembler.nrows if assembler.nrows is not None else dchi.nalldofs()
        import ctypes
        nnz = ctypes.c_int64()
        self.ctx.call("fs_stiffness", precision, assembler.mode, nrows, ctypes.byref(nnz))
        return self._fetch(nrows, nnz.value, assembler.csr)

    def mass(self, assembler, geom0, dchi=None):
        """mass(femm, assembler, geom0, dchi) -> lumped M."""
        if not isinstance(assembler, _Assembler):
            assembler, geom0, dchi = SysmatAssemblerSparseSymm(), assembler, geom0
        if not self._associatedgeometry:
            raise AssertionError("self._associatedgeometry == true")
        self._sync_inputs(geom0, dchi)
        nrows = assembler.nrows if assembler.nrows is not None else dchi.nalldofs()
        import ctypes
        nnz = ctypes.c_int64()
        self.ctx.call("fs_mass", assembler.mode, nrows, ctypes.byref(nnz))
        return self._fetch(nrows, nnz.value, assembler.csr)

    def restoringforce(self, geom0, u1, Rfield1, dchi, precision=FS_FP64):
        """-K U for the generalized displacements held in dchi.values (6 per node),
        returned as a vector of nalldofs(dchi) entries.  An extension: the
        reference shells have no restoringforce; its explicit loop subtracts
        E = K U (plate_expl_examples.jl:85)."""
        K_n = dchi.nalldofs()
        self.stiffness(SysmatAssemblerSparse(), geom0, u1, Rfield1, dchi, precision=precision)
        d = np.asarray(dchi.dofnums, dtype=np.int64)
        U = np.zeros(K_n)
        ok = (d >= 1) & (d <= K_n)
        U[d[ok] - 1] = np.asarray(dchi.values)[ok]
        F = np.zeros(K_n)
        self.ctx.call("fs_restoring_force", ptr(U), ptr(F))
        return F

    # quantity symbols of inspectintegpoints (src/FEMMShellT3FFModule.jl:893-902);
    # anything else (the default :Cauchy) reports the bending moments
    _RES_QUANTITY = {"bending": _abi.FS_RES_MOMENT, "moment": _abi.FS_RES_MOMENT,
                     "bending_moment": _abi.FS_RES_MOMENT, "transverse_shear": _abi.FS_RES_SHEAR,
                     "transverse": _abi.FS_RES_SHEAR, "shear": _abi.FS_RES_SHEAR,
                     "membrane_force": _abi.FS_RES_MEMBRANE, "membrane": _abi.FS_RES_MEMBRANE}

    def _point_locations(self, geom0):
        """Integration points: per point its element (0-based), its tangents
        (3x2) and its location, in the reference's point order."""
        X = np.asarray(geom0.values, dtype=np.float64)[self.conn - 1]  # nelem x nen x 3
        if self.nen == 3:
            tang = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]], axis=2)
            return np.arange(X.shape[0]), np.zeros(X.shape[0], dtype=np.int64), tang, X.mean(axis=1)
        gp = 0.577350269189626
        locs, tangs = [], []
        for j in range(4):
            xi, eta = (-gp if j < 2 else gp), (gp if j & 1 else -gp)
            N = np.array([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta), (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)]) / 4
            dxi = np.array([-(1 - eta), (1 - eta), (1 + eta), -(1 + eta)]) / 4
            deta = np.array([-(1 - xi), -(1 + xi), (1 + xi), (1 - xi)]) / 4
            locs.append(np.einsum("a,eac->ec", N, X))
            tangs.append(np.stack([np.einsum("a,eac->ec", dxi, X), np.einsum("a,eac->ec", deta, X)], axis=2))
        ne = X.shape[0]
        el = np.repeat(np.arange(ne), 4)
        qp = np.tile(np.arange(1, 5), ne)
        return el, qp, np.stack(tangs, axis=1).reshape(ne * 4, 3, 2), np.stack(locs, axis=1).reshape(ne * 4, 3)

    def resultants(self, geom0, u, quantity="bending", outputcsys=None):
        """Stress resultants at every integration point (npoints x 3): the
        values inspectintegpoints hands to its inspector, in double.  outputcsys:
        None (the element frame at the point: the default mcsys), a 3x3
        matrix, an (npoints, 3, 3) array, or a callable (XYZ, tangents, feid,
        qpid) -> 3x3 evaluated per point like updatecsmat!."""
        if not self._associatedgeometry:
            raise AssertionError("self._associatedgeometry == true")
        self._sync_inputs(geom0, None)
        q = self._RES_QUANTITY.get(str(quantity).lstrip(":"), _abi.FS_RES_MOMENT)
        uu = np.asfortranarray(u.values if hasattr(u, "values") else u, dtype=np.float64)
        if uu.shape != (geom0.values.shape[0], 6):
            raise ValueError("u must hold 6 values per node")
        npt = self.conn.shape[0] * (1 if self.nen == 3 else 4)
        if outputcsys is None:
            cs, ncs = None, 0
        elif callable(outputcsys):
            el, qp, tang, loc = self._point_locations(geom0)
            cs = np.stack([np.asarray(outputcsys(loc[k].reshape(1, 3), tang[k], el[k] + 1, qp[k]), dtype=np.float64)
                           for k in range(npt)])
            ncs = npt
        else:
            cs = np.asarray(outputcsys, dtype=np.float64)
            ncs = 1 if cs.ndim == 2 else cs.shape[0]
        csf = None if cs is None else np.ascontiguousarray(cs.reshape(-1, 3, 3).transpose(0, 2, 1))
        out = np.zeros((npt, 3))
        self.ctx.call("fs_resultants", q, ptr(uu), ptr(csf), ncs, ptr(out))
        return out

    def inspectintegpoints(self, geom0, u, felist, inspector, idat, quantity="Cauchy", outputcsys=None):
        """inspectintegpoints(femm, geom0, u, felist, inspector, idat, quantity;
        outputcsys) (src/FEMMShellT3FFModule.jl:850-962, src/FEMMShellQ4RSModule.jl:
        1061-1170): all points are evaluated on the GPU in one launch, then
        inspector(idat, i, conn, ecoords, out, loc) is called for every point of
        the elements of felist (1-based element numbers) in the reference's
        order, and the final idat is returned."""
        out = self.resultants(geom0, u, quantity, outputcsys)
        X = np.asarray(geom0.values, dtype=np.float64)
        el, qp, _, loc = self._point_locations(geom0)
        npe = 1 if self.nen == 3 else 4
        for i in felist:
            e = int(i) - 1
            for j in range(npe):
                k = e * npe + j
                idat = inspector(idat, int(i), self.conn[e], X[self.conn[e] - 1], out[k].copy(),
                                 loc[k].reshape(1, 3))
        return idat

    def fieldfromintegpoints(self, geom0, u, quantity, component, outputcsys=None):
        """fieldfromintegpoints(femm, geom0, u, quantity, component; outputcsys)
        of FinEtools with its default node-value method (inverse distance): each
        node's value is the average of the integration-point values of the
        elements that hold it, weighted by the inverse squared distance from
        the point to the node.  component: 1-based.  Returns nnodes values
        (zero at nodes of no element).  The points' values come from the GPU
        (fs_resultants), the weighting runs on the host."""
        vals = self.resultants(geom0, u, quantity, outputcsys)[:, int(component) - 1]
        X = np.asarray(geom0.values, dtype=np.float64)
        el, _, _, loc = self._point_locations(geom0)
        nodes = self.conn[el] - 1                                   # npoints x nen
        d2 = ((X[nodes] - loc[:, None, :]) ** 2).sum(axis=2)
        w = 1.0 / d2
        num = np.zeros(X.shape[0])
        den = np.zeros(X.shape[0])
        np.add.at(num, nodes.ravel(), (w * vals[:, None]).ravel())
        np.add.at(den, nodes.ravel(), w.ravel())
        return np.divide(num, den, out=np.zeros_like(num), where=den > 0)

    # -- extras ----------------------------------------------------------------
    def element_matrices(self, geom0, precision=FS_FP64):
        """All element stiffness matrices in the global basis (nelem x nd x nd);
        FS_MIXED_COMP's float pairs as the doubles nearest hi + lo."""
        self._sync_inputs(geom0, None)
        nd = 6 * self.nen
        out = np.zeros((self.conn.shape[0], nd, nd))
        self.ctx.call("fs_element_matrices", precision, ptr(out))
        return out.transpose(0, 2, 1).copy()

    def element_masses(self, geom0):
        self._sync_inputs(geom0, None)
        out = np.zeros((self.conn.shape[0], 2))
        self.ctx.call("fs_element_masses", ptr(out))
        return out

    def close(self):
        self.ctx.close()

    @classmethod
    def make(cls, fes, thickness, material, stab_fun=None, device=0):
        return cls(fes, thickness, material, stab_fun, device)


class FEMMShellT3FF(_FEMMShell):
    """src/FEMMShellT3FFModule.jl:101-112"""
    etype = _abi.FS_T3FF
    nen = 3
    default_stab = 5 / 12 / 1.5


class FEMMShellQ4RS(_FEMMShell):
    """src/FEMMShellQ4RSModule.jl:69-79"""
    etype = _abi.FS_Q4RS
    nen = 4
    default_stab = 0.1


class _FEMMShellComp(_FEMMShell):
    """Layered FEMM: `layup_groups` is a list of (fs_layup_group, element list
    1-based), as the reference's layup_groups field
    (src/FEMMShellT3FFCompModule.jl:63-77)."""

    def __init__(self, conn, layup_groups, stab_fun=None, device=0):
        if isinstance(layup_groups, _abi.fs_layup_group):
            layup_groups = [(layup_groups, np.arange(1, np.shape(conn)[0] + 1))]
        super().__init__(conn, 0.0, None, stab_fun, device, layup_groups)

    @classmethod
    def make(cls, fes, layup, stab_fun=None, device=0):
        return cls(fes, layup, stab_fun, device)


class FEMMShellT3FFComp(_FEMMShellComp):
    etype = _abi.FS_T3FFCOMP
    nen = 3
    default_stab = 5 / 12 / 1.5


class FEMMShellQ4RSComp(_FEMMShellComp):
    etype = _abi.FS_Q4RSCOMP
    nen = 4
    default_stab = 0.1


class ShellBatch:
    """Uneven homogeneous meshes of one shell family assembled together
    (fs_batch_*): one element launch over the work-list of all elements and
    one gather launch.  `meshes` is a list of (geom0, conn, dchi, thickness);
    each mesh's matrix equals what its own FEMM would return."""

    def __init__(self, femm_cls, meshes, material, stab_fun=None, nrows=None, device=0):
        import ctypes
        from .materials import shell_material_stiffness
        self.ctx = Context(device)
        Dps, Dt = shell_material_stiffness(material)
        quads = femm_cls.nen == 4
        p = _abi.make_params(Dps, Dt, material.massdensity(), 0.0,
                             stab_c=stab_coefficient(stab_fun, femm_cls.default_stab), quads=quads)
        self.ctx.call("fs_params_set", p, None)
        self.n = len(meshes)
        keep = []
        arr = lambda vals, t: (t * self.n)(*vals)
        xyzs = [np.asfortranarray(g.values, dtype=np.float64) for g, _, _, _ in meshes]
        conns = [np.ascontiguousarray(c, dtype=np.int64) for _, c, _, _ in meshes]
        dofs = [np.asfortranarray(d.dofnums, dtype=np.int64) for _, _, d, _ in meshes]
        keep += xyzs + conns + dofs
        self.nrows = [int(nrows[i]) if nrows is not None else d.nalldofs() for i, (_, _, d, _) in enumerate(meshes)]
        vp = ctypes.c_void_p
        self.ctx.call("fs_batch_set", femm_cls.etype, self.n,
                      arr([x.shape[0] for x in xyzs], ctypes.c_int64), arr([x.ctypes.data for x in xyzs], vp),
                      arr([c.shape[0] for c in conns], ctypes.c_int64), arr([c.ctypes.data for c in conns], vp),
                      arr([d.ctypes.data for d in dofs], vp), arr(self.nrows, ctypes.c_int64),
                      arr([float(t) for _, _, _, t in meshes], ctypes.c_double))
        self._keep = keep

    def stiffness(self, assembler=None, precision=FS_FP64, fetch=True):
        """All meshes' stiffness matrices (a list of scipy CSC, or CSR for
        SysmatAssemblerSparseCSRSymm)."""
        import ctypes
        import scipy.sparse as sp
        assembler = assembler or SysmatAssemblerSparseSymm()
        if not fetch:
            self.ctx.call("fs_batch_stiffness", precision, assembler.mode, None)
            return None
        nnz = (ctypes.c_int64 * self.n)()
        self.ctx.call("fs_batch_stiffness", precision, assembler.mode, nnz)
        out = []
        for i in range(self.n):
            n, z = self.nrows[i], nnz[i]
            colptr = np.empty(n + 1, dtype=np.int64)
            rowval = np.empty(z, dtype=np.int64)
            nzval = np.empty(z, dtype=np.float64)
            self.ctx.call("fs_batch_matrix_copy", i, ptr(colptr), ptr(rowval), ptr(nzval))
            cls = sp.csr_matrix if assembler.csr else sp.csc_matrix
            out.append(cls((nzval, rowval - 1, colptr - 1), shape=(n, n)))
        return out

    def close(self):
        self.ctx.close()

"""Host mirror of the reference co-rotational beam interface (FEMMCorotBeam).

Reference names and call pattern (FinEtoolsFlexStructures.jl 3.6.4):

    cs = CrossSectionRectangle(lambda s: b, lambda s: h, lambda s: [0, 1, 0])   # src/CrossSectionModule.jl
    xyz, conn, sections = merge_members([frame_member(X, n, cs), ...])          # src/MeshFrameMemberModule.jl
    femm = FEMMCorotBeam(conn, sections, MatDeforElastIso(E, nu, rho))
    K = femm.stiffness(geom0, u1, Rfield1, dchi)                                # src/FEMMCorotBeamModule.jl:972-1040
    M = femm.mass(geom0, u1, Rfield1, dchi, mass_type=...)                      # :810-881
    G = femm.gyroscopic(geom0, u1, Rfield1, v1, dchi)                           # :883-970
    Kg = femm.geostiffness(geom0, u1, Rfield1, dchi)                            # :1042-1110
    F = femm.restoringforce(geom0, u1, Rfield1, dchi)                           # :1112-1176
    F = femm.distribloads_global(geom0, u1, Rfield1, dchi, q)                   # :1186-1260

Matrices come back as scipy.sparse CSC matrices, vectors as numpy arrays of
nalldofs entries.  The element loops and the assembly run in
libflexshell.so on the GPU (double precision); the helpers for cross
sections, member meshes and rotation fields are host-side set-up code.
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import Context, InputCache, ptr
from .femm import NodalField, SysmatAssemblerSparseSymm, _Assembler

MASS_TYPE_CONSISTENT_NO_ROTATION_INERTIA = 0
MASS_TYPE_CONSISTENT_WITH_ROTATION_INERTIA = 1
MASS_TYPE_LUMPED_DIAGONAL_NO_ROTATION_INERTIA = 2
MASS_TYPE_LUMPED_DIAGONAL_WITH_ROTATION_INERTIA = 3


# ---------------------------------------------------------------------------
# rotations (src/RotUtilModule.jl and FinEtools rotmat3!/skewmat!)
# ---------------------------------------------------------------------------
def skewmat(v):
    """Skew matrix S with S x = v x x."""
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def rotmat3(a):
    """Rotation matrix of the rotation vector a (Rodrigues' formula)."""
    a = np.asarray(a, dtype=np.float64).reshape(3)
    na = np.sqrt(a @ a)
    if na == 0.0:
        return np.eye(3)
    u = a / na
    uu = np.outer(u, u)
    return np.cos(na) * (np.eye(3) - uu) + np.sin(na) / na * skewmat(a) + uu


def initial_Rfield(nnodes):
    """initial_Rfield (src/RotUtilModule.jl:16-22): identity rotation per node,
    stored as the 9 column-major entries of R in one row."""
    f = NodalField(np.zeros((nnodes, 9)))
    f.values[:, [0, 4, 8]] = 1.0
    return f


def update_rotation_field(Rfield, dchi):
    """update_rotation_field! (src/RotUtilModule.jl:29-42): R <- rotmat3(dtheta) R
    with the incremental rotations in columns 4:6 of dchi."""
    Rs = Rfield.values
    for i in range(Rs.shape[0]):
        R = Rs[i, :].reshape(3, 3, order="F")
        Rs[i, :] = (rotmat3(dchi.values[i, 3:6]) @ R).flatten(order="F")
    return Rfield


# ---------------------------------------------------------------------------
# interpolation (the Dierckx Spline1D calls of the reference, s = 0)
# ---------------------------------------------------------------------------
class _Interpolant:
    """Interpolating spline through (x, y) of degree k with smoothing 0.

    With k = len(x) - 1 (at most 3) it is the interpolating polynomial; with
    k = 3 and five or more points it is the cubic spline whose interior knots
    are x[2:-2] (FITPACK's knot choice for s = 0, i.e. the not-a-knot end
    conditions).  Outside [x[0], x[-1]] the end value is returned, as
    Spline1D's default bc = "nearest".
    """

    def __init__(self, x, y):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        self.x, self.y = x, y
        n = x.size
        if n < 2:
            raise ValueError("need at least two points")
        if n <= 4:
            # Newton divided differences of the interpolating polynomial
            c = y.copy()
            for j in range(1, n):
                c[j:] = (c[j:] - c[j - 1:-1]) / (x[j:] - x[:n - j])
            self.newton = c
            self.M = None
            return
        h = np.diff(x)
        A = np.zeros((n, n))
        r = np.zeros(n)
        # second derivatives M: interior continuity of the first derivative
        for i in range(1, n - 1):
            A[i, i - 1] = h[i - 1]
            A[i, i] = 2 * (h[i - 1] + h[i])
            A[i, i + 1] = h[i]
            r[i] = 6 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
        # not-a-knot: third derivative continuous at x[1] and x[n-2]
        A[0, 0], A[0, 1], A[0, 2] = h[1], -(h[0] + h[1]), h[0]
        A[n - 1, n - 3], A[n - 1, n - 2], A[n - 1, n - 1] = h[n - 2], -(h[n - 3] + h[n - 2]), h[n - 3]
        self.M = np.linalg.solve(A, r)
        self.newton = None

    def __call__(self, t):
        x, y = self.x, self.y
        t = float(min(max(t, x[0]), x[-1]))
        if self.M is None:
            c = self.newton
            v = c[-1]
            for j in range(c.size - 2, -1, -1):
                v = v * (t - x[j]) + c[j]
            return float(v)
        i = int(np.clip(np.searchsorted(x, t) - 1, 0, x.size - 2))
        h = x[i + 1] - x[i]
        a, b = x[i + 1] - t, t - x[i]
        M = self.M
        return float(M[i] * a ** 3 / (6 * h) + M[i + 1] * b ** 3 / (6 * h)
                     + (y[i] / h - M[i] * h / 6) * a + (y[i + 1] / h - M[i + 1] * h / 6) * b)


# torsion constant coefficient c(a/b) of a rectangle, J = c a b^3
# (table of src/CrossSectionModule.jl:143-158)
_RECT_RATIO = [1, 1.5, 2.0, 2.5, 3.0, 4.0, 5.0, 6.0, 10, 20, 40, 80, 200, 2000]
_RECT_COEF = [0.141, 0.196, 0.229, 0.249, 0.263, 0.281, 0.291, 0.299, 0.312, 0.317, 0.325, 0.33,
              1 / 3, 1 / 3]
_rect_torsion = _Interpolant(_RECT_RATIO, _RECT_COEF)


def _fn(v):
    return v if callable(v) else (lambda s, v=v: v)


# ---------------------------------------------------------------------------
# cross sections (src/CrossSectionModule.jl)
# ---------------------------------------------------------------------------
class CrossSectionCircle:
    """Solid circle: Bernoulli (no shear factor) or Timoshenko."""

    def __init__(self, radius, x1x2_vector, shear_resisting_area_factor=None):
        self.radius, self.x1x2 = _fn(radius), _fn(x1x2_vector)
        self.factor = shear_resisting_area_factor

    def parameters(self, s):
        R = self.radius(s)
        A = np.pi * R ** 2
        As = np.inf if self.factor is None else A * self.factor
        return dict(A=A, I1=np.pi / 2 * R ** 4, I2=np.pi / 4 * R ** 4, I3=np.pi / 4 * R ** 4,
                    J=np.pi / 2 * R ** 4, A2s=As, A3s=As,
                    x1x2_vector=np.asarray(self.x1x2(s), dtype=np.float64), dimensions=[R])


class CrossSectionHollowCircle:
    """Hollow circle (Bernoulli)."""

    def __init__(self, innerradius, outerradius, x1x2_vector):
        self.rint, self.rext, self.x1x2 = _fn(innerradius), _fn(outerradius), _fn(x1x2_vector)

    def parameters(self, s):
        Re, Ri = self.rext(s), self.rint(s)
        I2 = np.pi / 4 * (Re ** 4 - Ri ** 4)
        I3 = np.pi / 4 * (Re ** 4 - Ri ** 4)
        return dict(A=np.pi * (Re ** 2 - Ri ** 2), I1=I2 + I3, I2=I2, I3=I3,
                    J=np.pi / 2 * (Re ** 4 - Ri ** 4), A2s=np.inf, A3s=np.inf,
                    x1x2_vector=np.asarray(self.x1x2(s), dtype=np.float64), dimensions=[Re, Ri])


class CrossSectionRectangle:
    """Rectangle d2 x d3: Bernoulli (no shear factor) or Timoshenko."""

    def __init__(self, d2f, d3f, x1x2_vector, shear_resisting_area_factor=None):
        self.d2, self.d3, self.x1x2 = _fn(d2f), _fn(d3f), _fn(x1x2_vector)
        self.factor = shear_resisting_area_factor

    def parameters(self, s):
        d2, d3 = self.d2(s), self.d3(s)
        a, b = max(d2, d3), min(d2, d3)
        c = _rect_torsion(a / b)
        A = d2 * d3
        I2 = d2 * d3 ** 3 / 12
        I3 = d2 ** 3 * d3 / 12
        As = np.inf if self.factor is None else A * self.factor
        return dict(A=A, I1=I2 + I3, I2=I2, I3=I3, J=c * a * b ** 3, A2s=As, A3s=As,
                    x1x2_vector=np.asarray(self.x1x2(s), dtype=np.float64), dimensions=[d2, d3])


def section_array(params):
    """(nelem, 10) array A, I1, I2, I3, J, A2s, A3s, x1x2_vector from parameter dicts."""
    out = np.zeros((len(params), 10))
    for i, p in enumerate(params):
        out[i, :7] = [p["A"], p["I1"], p["I2"], p["I3"], p["J"], p["A2s"], p["A3s"]]
        out[i, 7:] = np.asarray(p["x1x2_vector"], dtype=np.float64).reshape(3)
    return out


# ---------------------------------------------------------------------------
# member meshes (src/MeshFrameMemberModule.jl)
# ---------------------------------------------------------------------------
def frame_member(xyz, nL, crosssection):
    """frame_member (src/MeshFrameMemberModule.jl:20-79): nL two-node elements
    on the curve through the vertices `xyz` (one per row), parameterised by
    the chord length.  Returns (node coordinates, 1-based conn, sections)."""
    X = np.asarray(xyz, dtype=np.float64)
    npts = X.shape[0]
    s = np.zeros(npts)
    for j in range(1, npts):
        s[j] = s[j - 1] + np.linalg.norm(X[j] - X[j - 1])
    itp = [_Interpolant(s, X[:, c]) for c in range(3)]
    t = np.linspace(0.0, s[-1], nL + 1)
    nodes = np.array([[itp[c](tt) for c in range(3)] for tt in t])
    if npts == 2:
        # the degree-1 spline is the straight segment
        nodes = X[0] + np.outer(t / s[-1], X[1] - X[0])
    conn = np.column_stack([np.arange(1, nL + 1), np.arange(2, nL + 2)]).astype(np.int64)
    # parameter of each element as the reference computes it (:46-56)
    h = np.linalg.norm(nodes[conn[:, 1] - 1] - nodes[conn[:, 0] - 1], axis=1)
    smid = np.zeros(nL)
    smid[0] = h[0] / 2
    stot = 0.0
    for i in range(1, nL):
        smid[i] = smid[i - 1] + h[i] / 2
        stot = smid[i] + h[i] / 2
    with np.errstate(divide="ignore", invalid="ignore"):
        params = [crosssection.parameters(smid[i] / stot) for i in range(nL)]
    return nodes, conn, section_array(params)


def merge_members(members, tolerance=0.001):
    """merge_members (src/MeshFrameMemberModule.jl:112-129): nodes closer than
    `tolerance` (in every coordinate) are fused, in order of first appearance;
    the elements are concatenated member by member."""
    xyz, conns, secs = [], [], []
    for nodes, conn, sec in members:
        base = []
        for p in nodes:
            hit = -1
            for k, q in enumerate(xyz):
                if np.all(np.abs(q - p) < tolerance):
                    hit = k
                    break
            if hit < 0:
                xyz.append(np.asarray(p, dtype=np.float64))
                hit = len(xyz) - 1
            base.append(hit + 1)
        base = np.asarray(base, dtype=np.int64)
        conns.append(base[np.asarray(conn, dtype=np.int64) - 1])
        secs.append(np.asarray(sec, dtype=np.float64))
    return np.array(xyz), np.vstack(conns), np.vstack(secs)


def selectnode(xyz, box, tolerance=0.0):
    """1-based nodes inside box [xmin xmax ymin ymax zmin zmax] inflated by tolerance."""
    b = np.asarray(box, dtype=np.float64).reshape(3, 2)
    X = np.asarray(xyz)
    ok = np.all((X >= b[:, 0] - tolerance) & (X <= b[:, 1] + tolerance), axis=1)
    return np.nonzero(ok)[0] + 1


# ---------------------------------------------------------------------------
# FEMM
# ---------------------------------------------------------------------------
class FEMMCorotBeam:
    """FEMMCorotBeam (src/FEMMCorotBeamModule.jl:23-56) on the GPU.

    conn: (nelem, 2) 1-based; sections: (nelem, 10) array (A, I1, I2, I3, J,
    A2s, A3s, x1x2_vector) as FESetL2Beam holds them; material: an object with
    E, nu and massdensity() (MatDeforElastIso)."""

    def __init__(self, conn, sections, material, device=0):
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        if self.conn.ndim != 2 or self.conn.shape[1] != 2:
            raise ValueError("connectivity must be nelem x 2")
        self.sections = np.ascontiguousarray(sections, dtype=np.float64)
        if self.sections.shape != (self.conn.shape[0], 10):
            raise ValueError("sections must be nelem x 10")
        self.material = material
        self.ctx = Context(device)
        self._geom = InputCache()
        self._dofs = InputCache()

    @property
    def nelem(self):
        return self.conn.shape[0]

    def _sync(self, geom0, u1, Rfield1, dchi, v1=None):
        xyz = np.asfortranarray(geom0.values, dtype=np.float64)
        if self._geom.copy is None or self._geom.copy.shape != xyz.shape:
            self.ctx.call("fs_mesh_set", _abi.FS_COROTBEAM, xyz.shape[0], ptr(xyz), self.nelem,
                          ptr(self.conn), None, None)
            secs = (_abi.fs_beam_section * self.nelem)()
            ctypes.memmove(secs, self.sections.ctypes.data, self.sections.nbytes)
            m = self.material
            self.ctx.call("fs_beam_setup", secs, float(m.E), float(m.nu), float(m.massdensity()))
            self._geom.store(xyz)
            self._dofs.clear()
        elif self._geom.stale(xyz):
            self.ctx.call("fs_geometry_set", ptr(xyz))
            self._geom.store(xyz)
        if dchi is not None:
            d = np.asfortranarray(dchi.dofnums, dtype=np.int64)
            if d.shape != (xyz.shape[0], 6):
                raise ValueError("dchi must have 6 dofs per node")
            if self._dofs.stale(d):
                self.ctx.call("fs_dofs_set", ptr(d))
                self._dofs.store(d)
        arr = lambda f, w: None if f is None else np.asfortranarray(
            np.asarray(getattr(f, "values", f), dtype=np.float64).reshape(xyz.shape[0], w, order="F"))
        u, R, v = arr(u1, 3), arr(Rfield1, 9), arr(v1, 6)
        self.ctx.call("fs_beam_state_set", ptr(u), ptr(R), ptr(v))

    def _matrix(self, which, assembler, dchi, mass_type=MASS_TYPE_CONSISTENT_WITH_ROTATION_INERTIA):
        import scipy.sparse as sp
        nrows = assembler.nrows if assembler.nrows is not None else dchi.nalldofs()
        nnz = ctypes.c_int64()
        self.ctx.call("fs_beam_matrix", which, mass_type, assembler.mode, nrows, ctypes.byref(nnz))
        colptr = np.empty(nrows + 1, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nzval = np.empty(nnz.value, dtype=np.float64)
        self.ctx.call("fs_matrix_copy", ptr(colptr), ptr(rowval), ptr(nzval))
        cls = sp.csr_matrix if assembler.csr else sp.csc_matrix
        return cls((nzval, rowval - 1, colptr - 1), shape=(nrows, nrows))

    @staticmethod
    def _split(args, n):
        """(assembler, *rest) with the default SysmatAssemblerSparseSymm when omitted."""
        if args and isinstance(args[0], _Assembler):
            return args[0], args[1:]
        return SysmatAssemblerSparseSymm(), args

    def stiffness(self, *args):
        """stiffness([assembler,] geom0, u1, Rfield1, dchi) (:972-1040)."""
        asm, (geom0, u1, Rfield1, dchi) = self._split(args, 4)
        self._sync(geom0, u1, Rfield1, dchi)
        return self._matrix(_abi.FS_BEAM_STIFFNESS, asm, dchi)

    def geostiffness(self, *args):
        """geostiffness([assembler,] geom0, u1, Rfield1, dchi) (:1042-1110)."""
        asm, (geom0, u1, Rfield1, dchi) = self._split(args, 4)
        self._sync(geom0, u1, Rfield1, dchi)
        return self._matrix(_abi.FS_BEAM_GEOSTIFFNESS, asm, dchi)

    def mass(self, *args, mass_type=MASS_TYPE_CONSISTENT_WITH_ROTATION_INERTIA):
        """mass([assembler,] geom0, u1, Rfield1, dchi; mass_type) (:810-881)."""
        asm, (geom0, u1, Rfield1, dchi) = self._split(args, 4)
        self._sync(geom0, u1, Rfield1, dchi)
        return self._matrix(_abi.FS_BEAM_MASS, asm, dchi, mass_type)

    def gyroscopic(self, *args, mass_type=MASS_TYPE_CONSISTENT_WITH_ROTATION_INERTIA):
        """gyroscopic([assembler,] geom0, u1, Rfield1, v1, dchi; mass_type) (:883-970)."""
        asm, (geom0, u1, Rfield1, v1, dchi) = self._split(args, 5)
        self._sync(geom0, u1, Rfield1, dchi, v1)
        return self._matrix(_abi.FS_BEAM_GYROSCOPIC, asm, dchi, mass_type)

    def restoringforce(self, *args):
        """restoringforce([assembler,] geom0, u1, Rfield1, dchi) (:1112-1176) -> vector."""
        _, (geom0, u1, Rfield1, dchi) = self._split(args, 4)
        self._sync(geom0, u1, Rfield1, dchi)
        F = np.zeros(dchi.nalldofs())
        self.ctx.call("fs_beam_restoringforce", F.size, ptr(F))
        return F

    def distribloads_global(self, *args):
        """distribloads_global([assembler,] geom0, u1, Rfield1, dchi, fi) (:1186-1260):
        fi is the force per unit length, one 3-vector or one per element."""
        _, (geom0, u1, Rfield1, dchi, fi) = self._split(args, 5)
        self._sync(geom0, u1, Rfield1, dchi)
        q = np.ascontiguousarray(fi, dtype=np.float64)
        per = 1 if q.ndim == 2 else 0
        F = np.zeros(dchi.nalldofs())
        self.ctx.call("fs_beam_distribloads_global", ptr(q), per, F.size, ptr(F))
        return F

    def element_matrices(self, which, geom0, u1=None, Rfield1=None, v1=None,
                         mass_type=MASS_TYPE_CONSISTENT_WITH_ROTATION_INERTIA):
        """All element matrices (nelem, 12, 12) of FS_BEAM_* `which`."""
        self._sync(geom0, u1, Rfield1, None, v1)
        out = np.zeros((self.nelem, 12, 12))
        self.ctx.call("fs_beam_element_matrices", which, mass_type, ptr(out))
        return out.transpose(0, 2, 1).copy()

    def element_vectors(self, which, geom0, u1=None, Rfield1=None, q=None):
        """Element restoring forces (which 4) or distributed loads (5), (nelem, 12)."""
        self._sync(geom0, u1, Rfield1, None)
        qa = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
        per = 1 if (qa is not None and qa.ndim == 2) else 0
        out = np.zeros((self.nelem, 12))
        self.ctx.call("fs_beam_element_vectors", which, ptr(qa), per, ptr(out))
        return out

    def close(self):
        self.ctx.close()

"""CPU oracle for the shell element-assembly hot path (TEST INFRASTRUCTURE).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module.  It wraps ``flexshell_oracle.c``, a plain-C
restatement of the reference (FinEtoolsFlexStructures.jl 3.6.4) element loops
and of the FinEtools 8.2.5 assembler semantics, and is never part of the
product path.

Parity pins: the oracle is checked against the reference's own known answers
(``tests/test_oracle_pins.py``): the NAFEMS FV12 free-plate frequencies
(test/test_shell_dynamics.jl:113-132, rtol 1e-6), the Scordelis-Lo roof
percentages for T3FF (test/test_shell_statics.jl:97-107) and Q4RS
(test/test_q4rs_shell_statics.jl:95-106), and the layup A-matrix values of
test/test_composite_layup.jl.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

T3FF, T3FFCOMP, Q4RS, Q4RSCOMP = 0, 1, 2, 3
RES_MOMENT, RES_SHEAR, RES_MEMBRANE = 1, 2, 3
CSYS_ISOPARAMETRIC, CSYS_CARTESIAN, CSYS_CYLINDRICAL, CSYS_SPHERICAL = 0, 1, 2, 3
KEEP_ZEROS, DROP_ZEROS, DIAG = 0, 1, 2

_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_i32_p = ctypes.POINTER(ctypes.c_int32)
_c_u8_p = ctypes.POINTER(ctypes.c_uint8)


SOURCES = ("flexshell_oracle.c", "corotbeam_oracle.c")
HEADERS = ("flexshell_oracle.h", "corotbeam_oracle.h")


def build(force=False):
    """Compile the oracle into oracle/_build/liboracle.so with gcc."""
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    deps = srcs + [os.path.join(HERE, f) for f in HEADERS]
    if (not force and os.path.exists(LIB_PATH)
            and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=c11", "-D_DEFAULT_SOURCE"] + srcs + ["-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class orc_params(ctypes.Structure):
    _fields_ = [
        ("etype", ctypes.c_int),
        ("Dps", ctypes.c_double * 9),
        ("Dt", ctypes.c_double * 4),
        ("rho", ctypes.c_double),
        ("thickness", _c_dbl_p),
        ("ngroups", ctypes.c_int),
        ("group", _c_i32_p),
        ("gA", _c_dbl_p), ("gB", _c_dbl_p), ("gD", _c_dbl_p),
        ("gH", _c_dbl_p), ("gcsmat", _c_dbl_p), ("gthick", _c_dbl_p),
        ("gmass", _c_dbl_p), ("gmoi", _c_dbl_p),
        ("stab_c", ctypes.c_double),
        ("drill_scale", ctypes.c_double),
        ("tsf", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_normals.restype = ctypes.c_int
        L.orc_normals_csys.restype = ctypes.c_int
        L.orc_assemble.restype = ctypes.c_int
        L.orc_result_nnz.restype = ctypes.c_int64
        L.orc_result_n.restype = ctypes.c_int64
        L.orc_all_element_stiffness.restype = ctypes.c_int
        L.orc_csc_accumulate_stiffness.restype = ctypes.c_int
        L.orc_cd_steps.restype = ctypes.c_int
        L.orc_cd_steps_load.restype = ctypes.c_int
        L.orc_laminate.restype = ctypes.c_int
        L.orc_assemble_elmats.restype = ctypes.c_int
        L.orc_beam_all.restype = ctypes.c_int
        L.orc_beam_element.restype = ctypes.c_int
        L.orc_beam_frame.restype = ctypes.c_double
        L.orc_resultants.restype = ctypes.c_int
        L.orc_distribloads.restype = ctypes.c_int
        L.orc_integration_points.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class Problem:
    """Inputs of one FEMM call in the reference's layouts.

    xyz: (nnodes,3) float64; conn: (nelem,nen) int64 1-based;
    dofnums: (nnodes,6) int64 1-based.  ``material`` is a dict with Dps (3x3),
    Dt (2x2), rho for the homogeneous types; ``groups`` a list of dicts with
    A,B,D (3x3), H (2x2), csmat (3x3), thickness, mass, moi for the layered
    types and ``group`` the per-element group index.
    """

    def __init__(self, etype, xyz, conn, dofnums=None, thickness=None, material=None,
                 groups=None, group=None, stab_c=None, drill_scale=1.0, tsf=0, order=None):
        self.etype = etype
        self.xyz = np.asfortranarray(xyz, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        self.nnodes = self.xyz.shape[0]
        self.nelem = self.conn.shape[0]
        self.dofnums = None if dofnums is None else np.asfortranarray(dofnums, dtype=np.int64)
        self.order = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
        p = orc_params()
        p.etype = etype
        if stab_c is None:
            stab_c = (5 / 12 / 1.5) if etype in (T3FF, T3FFCOMP) else 0.1
        p.stab_c = stab_c
        p.drill_scale = drill_scale
        p.tsf = tsf
        self._keep = []
        if etype in (T3FF, Q4RS):
            m = material
            p.Dps[:] = list(np.asarray(m["Dps"], dtype=np.float64).flatten(order="F"))
            p.Dt[:] = list(np.asarray(m["Dt"], dtype=np.float64).flatten(order="F"))
            p.rho = float(m.get("rho", 0.0))
            th = np.ascontiguousarray(np.broadcast_to(np.asarray(thickness, dtype=np.float64),
                                                      (self.nelem,)))
            self._keep.append(th)
            p.thickness = _p(th, _c_dbl_p)
        else:
            ng = len(groups)
            arr = {}
            for key, sz in (("A", 9), ("B", 9), ("D", 9), ("H", 4), ("csmat", 9)):
                arr[key] = np.ascontiguousarray(
                    np.concatenate([np.asarray(g[key], dtype=np.float64).flatten(order="F")
                                    for g in groups]))
            for key in ("thickness", "mass", "moi"):
                arr[key] = np.ascontiguousarray([float(g[key]) for g in groups], dtype=np.float64)
            gr = np.ascontiguousarray(group if group is not None else np.zeros(self.nelem),
                                      dtype=np.int32)
            self._keep.extend(list(arr.values()) + [gr])
            p.ngroups = ng
            p.group = _p(gr, _c_i32_p)
            p.gA, p.gB, p.gD = _p(arr["A"], _c_dbl_p), _p(arr["B"], _c_dbl_p), _p(arr["D"], _c_dbl_p)
            p.gH, p.gcsmat = _p(arr["H"], _c_dbl_p), _p(arr["csmat"], _c_dbl_p)
            p.gthick, p.gmass, p.gmoi = (_p(arr["thickness"], _c_dbl_p), _p(arr["mass"], _c_dbl_p),
                                         _p(arr["moi"], _c_dbl_p))
        self.params = p
        self.normals = None
        self.valid = None

    @property
    def nen(self):
        return self.conn.shape[1]

    def compute_normals(self, threshold_deg=30.0, csys_kind=0, csys_params=None):
        """associategeometry!: csys_kind 0 the isoparametric normals, 1
        cartesian (params: 3x3 matrix), 2 cylindrical (point on the axis, unit
        axis direction), 3 spherical (centre)."""
        nrm = np.zeros((self.nnodes, 3), dtype=np.float64, order="F")
        val = np.zeros(self.nnodes, dtype=np.uint8)
        prm = None if csys_params is None else np.ascontiguousarray(
            np.asarray(csys_params, dtype=np.float64).flatten(order="F"))
        st = lib().orc_normals_csys(self.etype, ctypes.c_int64(self.nnodes), _p(self.xyz, _c_dbl_p),
                                    ctypes.c_int64(self.nelem), _p(self.conn, _c_i64_p),
                                    _p(self.order, _c_i64_p), ctypes.c_double(threshold_deg),
                                    ctypes.byref(self.params), ctypes.c_int(csys_kind), _p(prm, _c_dbl_p),
                                    _p(nrm, _c_dbl_p), _p(val, _c_u8_p))
        assert st == 0
        self.normals, self.valid = nrm, val
        return nrm, val

    def set_normals(self, normals, valid):
        self.normals = np.asfortranarray(normals, dtype=np.float64)
        self.valid = np.ascontiguousarray(valid, dtype=np.uint8)

    def element_stiffness(self, nthreads=0):
        nd = 6 * self.nen
        out = np.zeros((self.nelem, nd, nd), dtype=np.float64)
        st = lib().orc_all_element_stiffness(
            ctypes.c_int64(self.nnodes), _p(self.xyz, _c_dbl_p), ctypes.c_int64(self.nelem),
            _p(self.conn, _c_i64_p), _p(self.normals, _c_dbl_p), _p(self.valid, _c_u8_p),
            ctypes.byref(self.params), ctypes.c_int(nthreads), _p(out, _c_dbl_p))
        if st != 0:
            raise RuntimeError("oracle element stiffness failed with status %d" % st)
        # stored column-major per element -> transpose to row-major view
        return np.ascontiguousarray(out.transpose(0, 2, 1))

    def resultants(self, u, quantity, cs=None):
        """Stress resultants at the integration points (inspectintegpoints):
        quantity RES_MOMENT, RES_SHEAR or RES_MEMBRANE; u (nnodes, 6); cs one
        3x3 csys matrix or one per point (npoints, 3, 3); None: the element
        frame at each point (the shells' default mcsys).
        Returns (npoints, 3), points in element order (Q4: four per element)."""
        npt = self.nelem * (1 if self.nen == 3 else 4)
        u = np.asfortranarray(u, dtype=np.float64)
        if cs is None:
            ncs, csf = 0, None
        else:
            cs = np.asarray(cs, dtype=np.float64)
            ncs = 1 if cs.ndim == 2 else cs.shape[0]
            csf = np.ascontiguousarray(cs.reshape(-1, 3, 3).transpose(0, 2, 1))  # column-major each
        out = np.zeros((npt, 3), dtype=np.float64)
        st = lib().orc_resultants(
            ctypes.c_int64(self.nnodes), _p(self.xyz, _c_dbl_p), ctypes.c_int64(self.nelem),
            _p(self.conn, _c_i64_p), _p(self.normals, _c_dbl_p), _p(self.valid, _c_u8_p),
            ctypes.byref(self.params), _p(u, _c_dbl_p), ctypes.c_int(quantity), _p(csf, _c_dbl_p),
            ctypes.c_int64(ncs), _p(out, _c_dbl_p))
        if st != 0:
            raise RuntimeError("oracle resultants failed with status %d" % st)
        return out

    def assemble(self, what="K", mode=KEEP_ZEROS, n=None, nthreads=0):
        """Returns (colptr, rowval, nzval) 1-based CSC arrays (== CSR for
        a symmetric matrix) and the matrix size."""
        if n is None:
            n = int(self.dofnums.max())
        res = ctypes.c_void_p()
        st = lib().orc_assemble(
            ctypes.c_int(0 if what == "K" else 1), ctypes.c_int(mode), ctypes.c_int64(self.nnodes),
            _p(self.xyz, _c_dbl_p), ctypes.c_int64(self.nelem), _p(self.conn, _c_i64_p),
            _p(self.order, _c_i64_p), _p(self.dofnums, _c_i64_p), ctypes.c_int64(n),
            _p(self.normals, _c_dbl_p), _p(self.valid, _c_u8_p), ctypes.byref(self.params),
            ctypes.c_int(nthreads), ctypes.byref(res))
        if st != 0:
            raise RuntimeError("oracle assembly failed with status %d" % st)
        L = lib()
        nnz = L.orc_result_nnz(res)
        colptr = np.zeros(n + 1, dtype=np.int64)
        rowval = np.zeros(nnz, dtype=np.int64)
        nzval = np.zeros(nnz, dtype=np.float64)
        L.orc_result_copy(res, _p(colptr, _c_i64_p), _p(rowval, _c_i64_p), _p(nzval, _c_dbl_p))
        L.orc_result_free(res)
        return colptr, rowval, nzval, n

    def stiffness_into_pattern(self, colptr, rowval, n=None, nthreads=0):
        """The oracle's element stiffness matrices summed into the values of
        a given 1-based CSC pattern (for meshes too large for the COO buffer
        of `assemble`).  Returns (vals, touched, missing): touched flags the
        stored entries that got a contribution, missing counts contributions
        outside the pattern."""
        if n is None:
            n = int(self.dofnums.max())
        colptr = np.ascontiguousarray(colptr, dtype=np.int64)
        rowval = np.ascontiguousarray(rowval, dtype=np.int64)
        vals = np.zeros(rowval.shape[0], dtype=np.float64)
        touched = np.zeros(rowval.shape[0], dtype=np.uint8)
        missing = ctypes.c_int64()
        st = lib().orc_csc_accumulate_stiffness(
            ctypes.c_int64(self.nnodes), _p(self.xyz, _c_dbl_p), ctypes.c_int64(self.nelem),
            _p(self.conn, _c_i64_p), _p(self.normals, _c_dbl_p), _p(self.valid, _c_u8_p),
            ctypes.byref(self.params), _p(self.dofnums, _c_i64_p), ctypes.c_int64(n),
            _p(colptr, _c_i64_p), _p(rowval, _c_i64_p), _p(vals, _c_dbl_p), _p(touched, _c_u8_p),
            ctypes.byref(missing), ctypes.c_int(nthreads))
        if st != 0:
            raise RuntimeError("oracle element stiffness failed with status %d" % st)
        return vals, touched, missing.value

    def assemble_scipy(self, what="K", mode=KEEP_ZEROS, n=None, nthreads=0):
        import scipy.sparse as sp
        colptr, rowval, nzval, n = self.assemble(what, mode, n, nthreads)
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(n, n))


def cd_steps(rowptr, colidx, vals, invMC, C, dt, nsteps, U, V, A, nthreads=0, Fmag=None, mul=None, step0=0):
    """Central-difference steps on a CSR stiffness (0-based rowptr/colidx);
    optional external force g(t) Fmag with mul[k] = g(k dt), the state at step
    index step0."""
    n = U.shape[0]
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    colidx = np.ascontiguousarray(colidx, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    for a in (U, V, A):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    Fm = None if Fmag is None else np.ascontiguousarray(Fmag, dtype=np.float64)
    mu = None if mul is None else np.ascontiguousarray(mul, dtype=np.float64)
    st = lib().orc_cd_steps_load(ctypes.c_int64(n), _p(rowptr, _c_i64_p), _p(colidx, _c_i64_p),
                                 _p(vals, _c_dbl_p), _p(np.ascontiguousarray(invMC), _c_dbl_p),
                                 _p(np.ascontiguousarray(C), _c_dbl_p), ctypes.c_double(dt),
                                 ctypes.c_int64(nsteps), _p(U, _c_dbl_p), _p(V, _c_dbl_p),
                                 _p(A, _c_dbl_p), _p(Fm, _c_dbl_p), _p(mu, _c_dbl_p),
                                 ctypes.c_int64(0 if mu is None else mu.shape[0]), ctypes.c_int64(step0),
                                 ctypes.c_int(nthreads))
    assert st == 0


def laminate(plies, offset=0.0, shear_model=0, tcf=0.0):
    """plies: list of dicts with Dps (3x3), Dts (2x2), thickness, angle (deg), rho."""
    k = len(plies)
    Dps = np.ascontiguousarray(np.concatenate([np.asarray(p["Dps"], float).flatten(order="F")
                                               for p in plies]))
    Dts = np.ascontiguousarray(np.concatenate([np.asarray(p["Dts"], float).flatten(order="F")
                                               for p in plies]))
    t = np.ascontiguousarray([p["thickness"] for p in plies], dtype=np.float64)
    ang = np.ascontiguousarray([p["angle"] for p in plies], dtype=np.float64)
    rho = np.ascontiguousarray([p.get("rho", 0.0) for p in plies], dtype=np.float64)
    A = np.zeros(9); B = np.zeros(9); D = np.zeros(9); H = np.zeros(4)
    md = ctypes.c_double(); mi = ctypes.c_double()
    lib().orc_laminate(ctypes.c_int(k), _p(Dps, _c_dbl_p), _p(Dts, _c_dbl_p), _p(t, _c_dbl_p),
                       _p(ang, _c_dbl_p), _p(rho, _c_dbl_p), ctypes.c_double(offset),
                       ctypes.c_int(shear_model), ctypes.c_double(tcf), _p(A, _c_dbl_p),
                       _p(B, _c_dbl_p), _p(D, _c_dbl_p), _p(H, _c_dbl_p), ctypes.byref(md),
                       ctypes.byref(mi))
    f = lambda a, s: a.reshape(s, order="F")
    return f(A, (3, 3)), f(B, (3, 3)), f(D, (3, 3)), f(H, (2, 2)), md.value, mi.value


# ---------------------------------------------------------------------------
# co-rotational beam (corotbeam_oracle.c)
# ---------------------------------------------------------------------------
BEAM_STIFFNESS, BEAM_GEOSTIFFNESS, BEAM_MASS, BEAM_GYROSCOPIC, BEAM_RESTORING, BEAM_DISTRIBLOAD = range(6)


def _result_arrays(res, n):
    L = lib()
    nnz = L.orc_result_nnz(res)
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowval = np.zeros(nnz, dtype=np.int64)
    nzval = np.zeros(nnz, dtype=np.float64)
    L.orc_result_copy(res, _p(colptr, _c_i64_p), _p(rowval, _c_i64_p), _p(nzval, _c_dbl_p))
    L.orc_result_free(res)
    return colptr, rowval, nzval


def assemble_elmats(Ke, conn, dofnums, n, mode=KEEP_ZEROS, order=None):
    """Assemble element matrices Ke (nelem, nd, nd) with the FinEtools
    assembler semantics; returns a scipy CSC matrix."""
    import scipy.sparse as sp
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    dofnums = np.asfortranarray(dofnums, dtype=np.int64)
    nelem, nen = conn.shape
    # column-major per element
    Kc = np.ascontiguousarray(np.asarray(Ke, dtype=np.float64).transpose(0, 2, 1))
    order = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    res = ctypes.c_void_p()
    st = lib().orc_assemble_elmats(ctypes.c_int(mode), ctypes.c_int(nen),
                                   ctypes.c_int64(dofnums.shape[0]), ctypes.c_int64(nelem),
                                   _p(conn, _c_i64_p), _p(order, _c_i64_p), _p(dofnums, _c_i64_p),
                                   ctypes.c_int64(n), _p(Kc, _c_dbl_p), ctypes.byref(res))
    assert st == 0
    colptr, rowval, nzval = _result_arrays(res, n)
    return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(n, n))


def assemble_vector(Fe, conn, dofnums, n):
    """SysvecAssembler: element vectors (nelem, 6 nen) summed in element order."""
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    dofnums = np.asfortranarray(dofnums, dtype=np.int64)
    Fe = np.ascontiguousarray(Fe, dtype=np.float64)
    F = np.zeros(n, dtype=np.float64)
    lib().orc_assemble_vector(ctypes.c_int64(dofnums.shape[0]), ctypes.c_int64(conn.shape[0]),
                              ctypes.c_int(conn.shape[1]), _p(conn, _c_i64_p), _p(dofnums, _c_i64_p),
                              ctypes.c_int64(n), _p(Fe, _c_dbl_p), _p(F, _c_dbl_p))
    return F


def _surface_args(xyz, conn):
    xyz = np.asfortranarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    return xyz, conn, ctypes.c_int(conn.shape[1]), ctypes.c_int64(xyz.shape[0]), ctypes.c_int64(conn.shape[0])


def npoints_of_rule(nen, rule):
    """Points per element: TriRule(npts) for triangles, GaussRule(2, order) for
    quadrilaterals, GaussRule(1, order) for two-node line elements."""
    return rule if nen in (2, 3) else rule * rule


def integration_points(xyz, conn, rule):
    """(nelem x npts, 9): location, x_xi, x_eta of every point, element order."""
    xyz, conn, nen, nn, ne = _surface_args(xyz, conn)
    out = np.zeros((conn.shape[0] * npoints_of_rule(conn.shape[1], rule), 9))
    st = lib().orc_integration_points(nen, nn, _p(xyz, _c_dbl_p), ne, _p(conn, _c_i64_p), ctypes.c_int(rule),
                                      _p(out, _c_dbl_p))
    if st != 0:
        raise RuntimeError("oracle integration_points failed with status %d" % st)
    return out


def distribloads(xyz, conn, dofnums, rule, m, force, n):
    """distribloads(FEMMBase(IntegDomain(fes, rule)), geom, P, fi, m) with the
    force given as one 6-vector, one per element or one per point."""
    xyz, conn, nen, nn, ne = _surface_args(xyz, conn)
    dofnums = np.asfortranarray(dofnums, dtype=np.int64)
    f = np.ascontiguousarray(force, dtype=np.float64).reshape(-1, 6)
    F = np.zeros(n, dtype=np.float64)
    st = lib().orc_distribloads(nen, nn, _p(xyz, _c_dbl_p), ne, _p(conn, _c_i64_p), _p(dofnums, _c_i64_p),
                                ctypes.c_int(rule), ctypes.c_int(m), _p(f, _c_dbl_p), ctypes.c_int64(f.shape[0]),
                                ctypes.c_int64(n), _p(F, _c_dbl_p))
    if st != 0:
        raise RuntimeError("oracle distribloads failed with status %d" % st)
    return F


class Beam:
    """Inputs of one FEMMCorotBeam call in the reference's layouts.

    xyz (nnodes,3); conn (nelem,2) 1-based; sections (nelem,10): A, I1, I2, I3,
    J, A2s, A3s, x1x2_vector; E, nu, rho of MatDeforElastIso.
    """

    def __init__(self, xyz, conn, sections, E, nu, rho=0.0):
        self.xyz = np.asfortranarray(xyz, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int64)
        self.sections = np.ascontiguousarray(sections, dtype=np.float64)
        assert self.sections.shape == (self.conn.shape[0], 10)
        self.E, self.nu, self.rho = float(E), float(nu), float(rho)

    @property
    def nnodes(self):
        return self.xyz.shape[0]

    @property
    def nelem(self):
        return self.conn.shape[0]

    def elements(self, which, u1=None, R1=None, v1=None, mass_type=1, q=None):
        """Element matrices (nelem,12,12) or vectors (nelem,12) of `which`."""
        nn = self.nnodes
        u1 = np.asfortranarray(u1 if u1 is not None else np.zeros((nn, 3)), dtype=np.float64)
        if R1 is None:
            R1 = np.tile(np.eye(3).flatten(order="F"), (nn, 1))
        R1 = np.asfortranarray(R1, dtype=np.float64)
        v1 = None if v1 is None else np.asfortranarray(v1, dtype=np.float64)
        vec = which in (BEAM_RESTORING, BEAM_DISTRIBLOAD)
        if q is not None:
            q = np.ascontiguousarray(np.broadcast_to(np.asarray(q, dtype=np.float64),
                                                     (self.nelem, 3)))
        out = np.zeros((self.nelem, 12 if vec else 144), dtype=np.float64)
        st = lib().orc_beam_all(ctypes.c_int(which), ctypes.c_int64(nn), _p(self.xyz, _c_dbl_p),
                                ctypes.c_int64(self.nelem), _p(self.conn, _c_i64_p),
                                _p(u1, _c_dbl_p), _p(R1, _c_dbl_p), _p(v1, _c_dbl_p),
                                _p(self.sections, _c_dbl_p), ctypes.c_double(self.E),
                                ctypes.c_double(self.nu), ctypes.c_double(self.rho),
                                ctypes.c_int(mass_type), _p(q, _c_dbl_p), _p(out, _c_dbl_p))
        assert st == 0
        if vec:
            return out
        return np.ascontiguousarray(out.reshape(self.nelem, 12, 12).transpose(0, 2, 1))

    def matrix(self, which, dofnums, n, mode=DROP_ZEROS, **kw):
        return assemble_elmats(self.elements(which, **kw), self.conn, dofnums, n, mode)

    def vector(self, which, dofnums, n, **kw):
        return assemble_vector(self.elements(which, **kw), self.conn, dofnums, n)

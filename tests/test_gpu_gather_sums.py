"""The gather's summation, value by value: every stored value is the sum of
its element contributions in ascending assembly rank (the order in which
Julia's sparse(I, J, V) combines duplicates) — a left-to-right double sum in
FP64, and in FS_MIXED the float-pair (TwoSum) accumulation of the float
contributions rounded once to double.  The expected values are
recomputed on the host from the library's own element matrices, so the
comparison is bitwise; in FS_MIXED_COMP the stored float pairs are summed
as float triples and rounded once, checked against the exact sum of the element
matrices as reported (each pair rounded to a double, which a pair whose low
half is far below its high half's last place does not fit exactly).  The
meshes exercise the single-batch path (Scordelis-Lo
roof, triangles and quadrilaterals) and the multi-batch path (a fan whose
centre node has more element pairs than one staging batch)."""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

import flexshell as F
import problems as PB
from test_gpu_parity import homog_pair

pytestmark = pytest.mark.gpu


def _contributions(Ke, conn, dof, n):
    """COO triplets (row, col, value) of the element matrices, element order."""
    rows, cols, vals = [], [], []
    for e in range(conn.shape[0]):
        d = dof[conn[e] - 1].ravel() - 1                       # node-major, 6 per node
        keep = np.nonzero(d < n)[0]
        ii, jj = np.meshgrid(keep, keep, indexing="ij")
        rows.append(d[ii].ravel())
        cols.append(d[jj].ravel())
        vals.append(Ke[e][ii, jj].ravel())
    return np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)


def _expected(Ke, conn, dof, n, precision):
    r, c, v = _contributions(Ke, conn, dof, n)
    order = np.lexsort((np.arange(r.size), c, r))             # by (row, col), then element order
    r, c, v = r[order], c[order], v[order]
    start = np.r_[0, np.nonzero((np.diff(r) != 0) | (np.diff(c) != 0))[0] + 1]
    size = np.diff(np.r_[start, r.size])
    if precision == F.FS_FP64:
        acc = v[start].copy()
        for k in range(1, size.max()):
            g = size > k
            acc[g] = acc[g] + v[start[g] + k]
        return r[start], c[start], acc
    v32 = v.astype(np.float32)
    assert np.array_equal(v32.astype(np.float64), v)          # the stored contributions are floats
    hi = v32[start].copy()
    lo = np.zeros_like(hi)
    for k in range(1, size.max()):
        g = size > k
        x = v32[start[g] + k]
        h = hi[g]
        t = h + x
        bp = t - h
        lo[g] = lo[g] + ((h - (t - bp)) + (x - bp))
        hi[g] = t
    return r[start], c[start], hi.astype(np.float64) + lo.astype(np.float64)


def _check_exact_sums(femm, geom0, dchi, conn, n):
    """FS_MIXED_COMP: every stored value within one unit in the last place of
    the exact sum of its element contributions as reported, plus the
    reported contributions' own rounding to double (half a unit in the last
    place of each; a float pair spans up to 24 + 24 bits and the gap between
    its halves) and what the float triple of the sum can lose (about 2^-72
    of the contributions' magnitudes)."""
    asm = F.SysmatAssemblerSparse() if n == dchi.nalldofs() else F.SysmatAssemblerFFBlock(n)
    K = femm.stiffness(asm, geom0, None, None, dchi, precision=F.FS_MIXED_COMP).tocoo()
    Ke = femm.element_matrices(geom0, F.FS_MIXED_COMP)
    r, c, v = _contributions(Ke, conn, dchi.dofnums, n)
    order = np.lexsort((np.arange(r.size), c, r))
    r, c, v = r[order], c[order], v[order]
    start = np.r_[0, np.nonzero((np.diff(r) != 0) | (np.diff(c) != 0))[0] + 1]
    stop = np.r_[start[1:], r.size]
    got = dict(zip(zip(K.row.tolist(), K.col.tolist()), K.data.tolist()))
    assert len(got) == start.size
    worst, info = 0.0, None
    for a, b in zip(start.tolist(), stop.tolist()):
        exact = sum((Fraction(x) for x in v[a:b].tolist()), Fraction(0))
        g = got[(int(r[a]), int(c[a]))]
        bound = Fraction(float(np.abs(v[a:b]).sum())) / 2 ** 52
        if exact != 0:
            bound += Fraction(float(np.spacing(abs(float(exact)))))
        q = float(abs(Fraction(g) - exact) / bound) if bound > 0 else float(g != 0.0)
        if q > worst:
            worst, info = q, (int(r[a]), int(c[a]), g, float(exact), v[a:b].tolist())
    assert worst <= 1.0, (n, worst, info)


def _check(femm, geom0, dchi, conn, n):
    _check_exact_sums(femm, geom0, dchi, conn, n)
    for precision in (F.FS_FP64, F.FS_MIXED):
        asm = F.SysmatAssemblerSparse() if n == dchi.nalldofs() else F.SysmatAssemblerFFBlock(n)
        K = femm.stiffness(asm, geom0, None, None, dchi, precision=precision).tocoo()
        Ke = femm.element_matrices(geom0, precision)
        er, ec, ev = _expected(Ke, conn, dchi.dofnums, n, precision)
        got = dict(zip(zip(K.row.tolist(), K.col.tolist()), K.data.tolist()))
        assert len(got) == er.size
        exp = np.array([got[(a, b)] for a, b in zip(er.tolist(), ec.tolist())])
        assert np.array_equal(exp, ev), (precision, np.abs(exp - ev).max())


@pytest.mark.parametrize("quads", [False, True])
def test_sums_in_assembly_order_roof(quads):
    d = PB.scordelis_lo(quads, 8)
    P, femm, geom0, dchi = homog_pair(d, quads)
    _check(femm, geom0, dchi, d["conn"], dchi.nalldofs())
    _check(femm, geom0, dchi, d["conn"], d["nfree"])
    femm.close()


def test_sums_in_assembly_order_fan():
    # 12 triangles around one node: 12 element pairs, more than the 8 the
    # gather stages at once
    m = 12
    ang = np.linspace(0, 2 * np.pi, m, endpoint=False)
    xyz = np.r_[[[0.0, 0.0, 0.0]], np.c_[np.cos(ang), np.sin(ang), 0.05 * np.sin(2 * ang)],
                1.7 * np.c_[np.cos(ang + 0.2), np.sin(ang + 0.2), 0.0 * ang]]
    conn = [[1, 2 + k, 2 + (k + 1) % m] for k in range(m)]
    conn += [[2 + k, 2 + m + k, 2 + (k + 1) % m] for k in range(m)]
    conn = np.array(conn)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.setebc([2 + m], 1)
    dchi.numberdofs()
    mat = F.materials.MatDeforElastIso(2.0e11, 0.3, 7850.0)
    femm = F.FEMMShellT3FF(conn, 0.01, mat)
    geom0 = F.NodalField(xyz)
    femm.associategeometry(geom0)
    _check(femm, geom0, dchi, conn, dchi.nalldofs())
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_pairs_summed_once_or_by_both_nodes_agree(quads):
    # the gather's two modes (each node-block pair summed by the lower node and
    # copied transposed, or summed by both nodes) store bitwise the same values
    d = PB.scordelis_lo(quads, 12)
    P, femm, geom0, dchi = homog_pair(d, quads)
    for n in (dchi.nalldofs(), d["nfree"]):
        asm = F.SysmatAssemblerSparse() if n == dchi.nalldofs() else F.SysmatAssemblerFFBlock(n)
        for prec in (F.FS_FP64, F.FS_MIXED, F.FS_MIXED_COMP):
            femm.ctx.call("fs_autotune", 0)
            K0 = femm.stiffness(asm, geom0, None, None, dchi, precision=prec)
            femm.ctx.call("fs_autotune", 3)
            K3 = femm.stiffness(asm, geom0, None, None, dchi, precision=prec)
            out = (ctypes.c_int32 * 4)()
            femm.ctx.call("fs_tuning_ex", out, 4)
            assert out[3] == 0
            assert np.array_equal(K0.indptr, K3.indptr) and np.array_equal(K0.indices, K3.indices)
            assert np.array_equal(K0.data, K3.data)
    femm.ctx.call("fs_autotune", 1)
    femm.close()

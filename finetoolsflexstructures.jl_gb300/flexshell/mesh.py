"""Mesh and field helpers that prepare inputs the way FinEtools does.

These mirror the FinEtools (8.2.5) helpers the reference tests and examples
use to build inputs for the hot path: ``T3block``/``Q4block`` structured
meshes, ``xyz3``, ``selectnode`` with a box, ``numberdofs!``.  They are host
helpers for tests and benchmarks; the hot path takes the arrays they produce.
"""
import numpy as np


def linearspace(a, b, n):
    return np.linspace(a, b, n)


def T3blockx(xs, ys, orientation="a"):
    """Triangles of a tensor-product grid (FinEtools T3blockx).  Nodes are
    numbered with x fastest; element pairs are produced with the x index
    outermost.  Orientation ``a`` splits each quad along the diagonal from
    (i+1, j) to (i, j+1)."""
    xs = np.asarray(xs, dtype=np.float64)
    ys = np.asarray(ys, dtype=np.float64)
    nL, nW = len(xs) - 1, len(ys) - 1
    X, Y = np.meshgrid(xs, ys)  # (nW+1, nL+1), x fastest when raveled
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    conn = np.zeros((2 * nL * nW, 3), dtype=np.int64)
    i = np.repeat(np.arange(1, nL + 1), nW)
    j = np.tile(np.arange(1, nW + 1), nL)
    f = (j - 1) * (nL + 1) + i
    if orientation == "a":
        conn[0::2] = np.stack([f, f + 1, f + (nL + 1)], axis=1)
        conn[1::2] = np.stack([f + 1, f + 1 + (nL + 1), f + (nL + 1)], axis=1)
    elif orientation == "b":
        conn[0::2] = np.stack([f, f + 1, f + 1 + (nL + 1)], axis=1)
        conn[1::2] = np.stack([f, f + 1 + (nL + 1), f + (nL + 1)], axis=1)
    else:
        raise ValueError("orientation must be 'a' or 'b'")
    return xy, conn


def T3block(rL, rW, nL, nW, orientation="a"):
    return T3blockx(linearspace(0.0, rL, nL + 1), linearspace(0.0, rW, nW + 1), orientation)


def Q4blockx(xs, ys):
    """Quadrilaterals of a tensor-product grid (FinEtools Q4blockx):
    counterclockwise [f, f+1, f+nL+2, f+nL+1], x index outermost."""
    xs = np.asarray(xs, dtype=np.float64)
    ys = np.asarray(ys, dtype=np.float64)
    nL, nW = len(xs) - 1, len(ys) - 1
    X, Y = np.meshgrid(xs, ys)
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    i = np.repeat(np.arange(1, nL + 1), nW)
    j = np.tile(np.arange(1, nW + 1), nL)
    f = (j - 1) * (nL + 1) + i
    conn = np.stack([f, f + 1, f + (nL + 1) + 1, f + (nL + 1)], axis=1).astype(np.int64)
    return xy, conn


def Q4block(rL, rW, nL, nW):
    return Q4blockx(linearspace(0.0, rL, nL + 1), linearspace(0.0, rW, nW + 1))


def xyz3(xy):
    xy = np.asarray(xy, dtype=np.float64)
    out = np.zeros((xy.shape[0], 3))
    out[:, : xy.shape[1]] = xy
    return out


def selectnode(xyz, box, inflate=0.0):
    """1-based indexes of nodes inside an axis-aligned box
    [xmin xmax ymin ymax zmin zmax] grown by ``inflate``."""
    xyz = np.asarray(xyz)
    box = np.asarray(box, dtype=np.float64).reshape(-1, 2)
    ok = np.ones(xyz.shape[0], dtype=bool)
    for d in range(box.shape[0]):
        ok &= (xyz[:, d] >= box[d, 0] - inflate) & (xyz[:, d] <= box[d, 1] + inflate)
    return np.nonzero(ok)[0] + 1


def numberdofs(is_fixed):
    """FinEtools numberdofs!: free dofs first (node-major, then component),
    fixed dofs numbered after them.  Returns (dofnums (nnodes,ndof) 1-based,
    nfreedofs)."""
    is_fixed = np.asarray(is_fixed, dtype=bool)
    flat = is_fixed.ravel()  # node-major order
    dof = np.zeros(flat.shape[0], dtype=np.int64)
    free = ~flat
    nfree = int(free.sum())
    dof[free] = np.arange(1, nfree + 1)
    dof[flat] = np.arange(nfree + 1, flat.shape[0] + 1)
    return dof.reshape(is_fixed.shape), nfree


def jittered_plate_q(n, side=1.0, jitter=0.2, seed=0, zfun=None):
    """Unit-square n x n quad grid with interior nodes jittered in-plane by
    U(+-jitter*h) (PCG64 stream of ``seed``), optional z = zfun(x, y)."""
    xy, conn = Q4block(side, side, n, n)
    h = side / n
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.uniform(-jitter * h, jitter * h, size=xy.shape)
    x, y = xy[:, 0], xy[:, 1]
    interior = (x > 1e-12 * side) & (x < side * (1 - 1e-12)) & (y > 1e-12 * side) & (y < side * (1 - 1e-12))
    xy = xy + d * interior[:, None]
    xyz = xyz3(xy)
    if zfun is not None:
        xyz[:, 2] = zfun(xyz[:, 0], xyz[:, 1])
    return xyz, conn


def quads_to_triangles(conn_q):
    """Split each quad [a b c d] into [a b d] and [b c d] (the T3block 'a'
    diagonal), element pairs kept adjacent."""
    conn_q = np.asarray(conn_q, dtype=np.int64)
    t = np.empty((2 * conn_q.shape[0], 3), dtype=np.int64)
    t[0::2] = conn_q[:, [0, 1, 3]]
    t[1::2] = conn_q[:, [1, 2, 3]]
    return t


def Q4toT3(conn_q, orientation="default"):
    """FinEtools Q4toT3: each quad [a b c d] becomes [a b c] and [a c d]
    (``"alternate"``: [a b d] and [c d b]), the two triangles of a quad
    adjacent in the element order."""
    conn_q = np.asarray(conn_q, dtype=np.int64)
    l1, l2 = ((0, 1, 2), (0, 2, 3)) if orientation == "default" else ((0, 1, 3), (2, 3, 1))
    t = np.empty((2 * conn_q.shape[0], 3), dtype=np.int64)
    t[0::2] = conn_q[:, l1]
    t[1::2] = conn_q[:, l2]
    return t


def meshboundary(conn):
    """Boundary of a triangle or quadrilateral mesh: the two-node edges that
    belong to one element only (nedges x 2, 1-based), each with the
    orientation it has in its element, in the order of the elements and of
    their edges (node 1-2, 2-3, ...)."""
    conn = np.asarray(conn, dtype=np.int64)
    nen = conn.shape[1]
    edges = np.stack([conn[:, [k, (k + 1) % nen]] for k in range(nen)], 1).reshape(-1, 2)
    key = np.sort(edges, 1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    return edges[cnt[inv.ravel()] == 1]


def selectelem(xyz, conn, box, inflate=0.0):
    """0-based indexes of the elements whose nodes all lie inside the box
    [xmin xmax ymin ymax zmin zmax] grown by ``inflate`` (FinEtools
    selectelem with ``box`` and ``allin = true``)."""
    inside = np.zeros(np.asarray(xyz).shape[0] + 1, dtype=bool)
    inside[selectnode(xyz, box, inflate)] = True
    return np.nonzero(inside[np.asarray(conn, dtype=np.int64)].all(1))[0]


def mergenodes(xyz, conn, tolerance):
    """FinEtools mergenodes: nodes closer than ``tolerance`` to an earlier
    node become that node; the remaining nodes keep their order.  Returns the
    new coordinates and connectivity (1-based)."""
    from scipy.spatial import cKDTree
    xyz = np.asarray(xyz, dtype=np.float64)
    rep = np.arange(xyz.shape[0])
    for i, j in sorted(cKDTree(xyz).query_pairs(tolerance)):
        rep[max(i, j)] = min(rep[i], rep[j])
    keep = rep == np.arange(rep.shape[0])
    num = np.cumsum(keep)[rep]  # 1-based number of each node's survivor
    return xyz[keep], num[np.asarray(conn, dtype=np.int64) - 1]

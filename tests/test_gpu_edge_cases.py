"""Edge cases of the assembly on the GPU, against the oracle: one element,
nodes that no element uses, an empty mesh, every dof fixed, a node whose row
is longer than the gather keeps in registers (the in-place path), an
element order that is not the mesh order, the entry points that need the
last matrix to be a stiffness, the end of the explicit state at a new
assembly, and the batch copy of a current matrix that is not the batch's.  FP64 within 1e-12 of the oracle with the
identical pattern; mixed within 1e-6."""
import numpy as np
import pytest

import flexshell as F
from flexshell import _abi
from oracle import oracle as O
from checks import relmax, same_pattern
from test_gpu_parity import _Mat

pytestmark = pytest.mark.gpu

E, NU, T = 2.0e11, 0.3, 0.01
DPS = E / (1 - NU ** 2) * np.array([[1, NU, 0], [NU, 1, 0], [0, 0, (1 - NU) / 2]])
MAT = dict(Dps=DPS, Dt=E / 2 / (1 + NU) * np.eye(2), rho=7850.0)


def _pair(xyz, conn, fixed_nodes=()):
    quads = conn.shape[1] == 4
    f = F.NodalField(np.zeros((xyz.shape[0], 6)))
    for c in range(1, 7):
        if len(fixed_nodes):
            f.setebc(fixed_nodes, c)
    f.numberdofs()
    et = O.Q4RS if quads else O.T3FF
    stab = 0.1 if quads else 5 / 12 / 1.5
    P = O.Problem(et, xyz, conn, f.dofnums, thickness=T, material=MAT, stab_c=stab)
    P.compute_normals()
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(conn, T, _Mat(MAT), stab_fun=stab)
    geom0 = F.NodalField(xyz)
    femm.associategeometry(geom0)
    return P, femm, geom0, f


def _check(P, femm, geom0, dchi, n=None):
    n = dchi.nalldofs() if n is None else n
    asm = F.SysmatAssemblerSparse() if n == dchi.nalldofs() else F.SysmatAssemblerFFBlock(n)
    K = femm.stiffness(asm, geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS, n=n)
    assert K.shape == Ko.shape and same_pattern(K, Ko)
    if Ko.nnz:
        assert relmax(K, Ko) <= 1e-12
        Km = femm.stiffness(asm, geom0, None, None, dchi, precision=F.FS_MIXED)
        assert same_pattern(Km, Ko) and relmax(Km, Ko) <= 1e-6
    return K


@pytest.mark.parametrize("quads", [False, True])
def test_single_element(quads):
    xyz = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.05], [0.9, 1.2, -0.02], [-0.1, 0.8, 0.03]])
    conn = np.array([[1, 2, 3, 4]] if quads else [[1, 2, 3]])
    if not quads:
        xyz = xyz[:3]
    P, femm, geom0, dchi = _pair(xyz, conn)
    K = _check(P, femm, geom0, dchi)
    assert K.nnz == (6 * conn.shape[1]) ** 2
    femm.close()


def test_unused_nodes_keep_empty_rows():
    # a 4 x 4 quad patch split into triangles, plus three nodes no element uses
    n = 4
    xs, ys = np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    xyz = np.c_[xs.ravel(), ys.ravel(), 0.02 * np.sin(3 * xs.ravel())]
    idx = lambda i, j: i * (n + 1) + j + 1
    conn = []
    for i in range(n):
        for j in range(n):
            conn += [[idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)], [idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)]]
    conn = np.array(conn)
    xyz = np.r_[xyz, [[2.0, 2.0, 0.0], [3.0, 2.0, 0.0], [2.0, 3.0, 0.0]]]
    P, femm, geom0, dchi = _pair(xyz, conn)
    K = _check(P, femm, geom0, dchi)
    orphan = dchi.dofnums[-3:].ravel() - 1
    Kc = K.tocsc()
    assert all(Kc.indptr[d + 1] == Kc.indptr[d] for d in orphan)
    femm.close()


def test_empty_mesh_and_all_dofs_fixed():
    xyz = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    # every dof fixed: the free-free block is empty
    P, femm, geom0, dchi = _pair(xyz, np.array([[1, 2, 3]]), fixed_nodes=[1, 2, 3])
    assert dchi.nfreedofs == 0
    K = femm.stiffness(F.SysmatAssemblerFFBlock(0), geom0, None, None, dchi)
    assert K.shape == (0, 0) and K.nnz == 0
    femm.close()
    # no elements at all: an all-zero matrix of the requested size
    import ctypes
    from flexshell._lib import ptr
    ctx = F.Context(0)
    conn = np.zeros((0, 3), dtype=np.int64)
    xyzf = np.asfortranarray(xyz)
    dof = np.asfortranarray(np.arange(1, 19, dtype=np.int64).reshape(3, 6))
    ctx.call("fs_mesh_set", _abi.FS_T3FF, 3, ptr(xyzf), 0, ptr(conn), None, ptr(dof))
    prm = _abi.make_params(DPS, MAT["Dt"], MAT["rho"], T, stab_c=5 / 12 / 1.5)
    ctx.call("fs_params_set", prm, None)
    ctx.call("fs_normals_compute")
    nnz = ctypes.c_int64(-1)
    ctx.call("fs_stiffness", _abi.FS_FP64, _abi.FS_ASM_SPARSE, 18, ctypes.byref(nnz))
    assert nnz.value == 0
    colptr = np.zeros(19, dtype=np.int64)
    ctx.call("fs_matrix_copy", ptr(colptr), None, None)
    assert np.all(colptr == 1)
    ctx.close()


def test_node_with_more_pairs_than_one_staging_batch():
    # a fan of 10 triangles: the centre node has 10 element pairs, more than the
    # 8 the gather stages at once, and a row of 66 columns kept in registers
    m = 10
    ang = np.linspace(0, 2 * np.pi, m, endpoint=False)
    xyz = np.r_[[[0.0, 0.0, 0.0]], np.c_[np.cos(ang), np.sin(ang), 0.05 * np.sin(2 * ang)]]
    conn = np.array([[1, 2 + k, 2 + (k + 1) % m] for k in range(m)])
    P, femm, geom0, dchi = _pair(xyz, conn)
    K = _check(P, femm, geom0, dchi)
    assert K.tocsr()[dchi.dofnums[0, 0] - 1].nnz == 66
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_long_rows_take_the_in_place_path(quads):
    # a fan of 48 triangles (or 12 quads with 30 degree corners) around one
    # centre node: the centre's row holds 49 (or 25) nodes x 6 = 294 (or 150)
    # columns, above the 128 a warp keeps in registers
    m = 24 if quads else 48
    ang = np.linspace(0, 2 * np.pi, m, endpoint=False)
    if quads:
        ring1 = np.c_[0.5 * np.cos(ang), 0.5 * np.sin(ang), 0.02 * np.cos(2 * ang)]
        xyz = np.r_[[[0.0, 0.0, 0.0]], ring1]
        # quads (centre, k, k+1, k+2) for even k: every ring node touches the centre
        conn = np.array([[1, 2 + k, 2 + (k + 1) % m, 2 + (k + 2) % m] for k in range(0, m, 2)])
    else:
        ring = np.c_[np.cos(ang), np.sin(ang), 0.05 * np.sin(3 * ang)]
        xyz = np.r_[[[0.0, 0.0, 0.0]], ring]
        conn = np.array([[1, 2 + k, 2 + (k + 1) % m] for k in range(m)])
    P, femm, geom0, dchi = _pair(xyz, conn)
    K = _check(P, femm, geom0, dchi)
    d0 = dchi.dofnums[0, 0] - 1
    assert K.tocsr()[d0].nnz > 128
    femm.close()


def test_element_order_not_the_mesh_order():
    # elements listed in a shuffled order: the assembly follows the given order
    n = 6
    xs, ys = np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    rng = np.random.default_rng(9)
    xyz = np.c_[xs.ravel(), ys.ravel(), 0.01 * rng.normal(size=xs.size)]
    idx = lambda i, j: i * (n + 1) + j + 1
    conn = np.array([[idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
                     for i in range(n) for j in range(n)])
    conn = conn[rng.permutation(conn.shape[0])]
    conn = np.array([np.roll(c, rng.integers(4)) for c in conn])  # varied local numbering
    P, femm, geom0, dchi = _pair(xyz, conn, fixed_nodes=[1, 2, 3])
    _check(P, femm, geom0, dchi)
    _check(P, femm, geom0, dchi, n=dchi.nfreedofs)
    femm.close()


def test_last_stiffness_entry_points_refuse_another_matrix():
    # fs_explicit_setup, fs_power_iteration, fs_restoring_force and
    # fs_shift_factor use the last matrix assembled, which must be a
    # stiffness: after fs_mass each returns FS_ERR_STATE (before any launch);
    # after fs_stiffness again they run
    import ctypes
    import problems as PB
    from flexshell import materials
    from flexshell._lib import FlexShellError, ptr
    xyz, conn, dof, nfree = PB.jittered_plate(4, False, seed=1)
    femm = F.FEMMShellT3FF(conn, 0.01, materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    m = np.ascontiguousarray(
        femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi).diagonal())
    invm, c, u, f = 1.0 / m, np.zeros(nfree), np.ones(nfree), np.zeros(nfree)
    om, kd = ctypes.c_double(), ctypes.c_int64()
    calls = [("fs_explicit_setup", (F.FS_FP64, ptr(invm), ptr(c), ctypes.c_double(1e-6))),
             ("fs_power_iteration", (ptr(m), ctypes.c_int64(5), ctypes.c_uint64(1), ctypes.byref(om))),
             ("fs_restoring_force", (ptr(u), ptr(f))),
             ("fs_shift_factor", (ctypes.c_double(0.0), ptr(m), ctypes.byref(kd)))]
    for name, args in calls:
        with pytest.raises(FlexShellError) as e:
            femm.ctx.call(name, *args)
        assert e.value.code == _abi.FS_ERR_STATE, name
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    for name, args in calls[:3]:
        femm.ctx.call(name, *args)
    assert om.value > 0 and np.abs(f).max() > 0
    femm.close()


def test_explicit_state_ends_with_a_new_assembly():
    # the captured explicit steps read the pattern and, in the CSR form, the
    # current matrix: an assembly after fs_explicit_setup ends the state, so
    # the next run is refused (FS_ERR_STATE) instead of reading buffers that
    # the assembly may have replaced; a new setup starts it again
    import ctypes
    import problems as PB
    from flexshell import materials
    from flexshell._lib import FlexShellError, ptr
    xyz, conn, dof, nfree = PB.jittered_plate(4, True, seed=2)
    femm = F.FEMMShellQ4RS(conn, 0.01, materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    m = np.ascontiguousarray(
        femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi).diagonal())
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    invm, c, v0 = 1.0 / m, np.zeros(nfree), np.full(nfree, 1e-3)
    z, u = np.zeros(nfree), np.zeros(nfree)
    ctx = femm.ctx
    ctx.call("fs_explicit_setup", F.FS_FP64, ptr(invm), ptr(c), ctypes.c_double(1e-7))
    ctx.call("fs_explicit_set_state", ptr(z), ptr(v0), ptr(z))
    ctx.call("fs_explicit_run", ctypes.c_int64(64))
    femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi)
    for name, args in (("fs_explicit_run", (ctypes.c_int64(64),)),
                       ("fs_explicit_get_state", (ptr(u), None, None))):
        with pytest.raises(FlexShellError) as e:
            ctx.call(name, *args)
        assert e.value.code == _abi.FS_ERR_STATE, name
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    ctx.call("fs_explicit_setup", F.FS_FP64, ptr(invm), ptr(c), ctypes.c_double(1e-7))
    ctx.call("fs_explicit_set_state", ptr(z), ptr(v0), ptr(z))
    ctx.call("fs_explicit_run", ctypes.c_int64(64))
    ctx.call("fs_explicit_get_state", ptr(u), None, None)
    assert np.abs(u).max() > 0
    femm.close()


def test_batch_copy_refuses_another_current_matrix():
    # the batch copy slices the current matrix at the meshes' row offsets:
    # after a matrix of another size is assembled in the batch's context it
    # is refused (FS_ERR_STATE) instead of reading past that matrix's rows
    import ctypes
    import problems as PB
    from flexshell import materials
    from flexshell._lib import FlexShellError, ptr
    meshes = []
    for k, n in enumerate([3, 4]):
        xyz, conn, dof, nfree = PB.jittered_plate(n, False, seed=k)
        dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
        dchi.dofnums = np.asfortranarray(dof)
        meshes.append((F.NodalField(xyz), conn, dchi, 0.01))
    b = F.ShellBatch(F.FEMMShellT3FF, meshes, materials.MatDeforElastIso(2.0e11, 0.3, 7850.0))
    Ks = b.stiffness(F.SysmatAssemblerSparse())
    total = sum(b.nrows)
    nnz = ctypes.c_int64()
    b.ctx.call("fs_mass", _abi.FS_ASM_DIAG, ctypes.c_int64(total - 6), ctypes.byref(nnz))
    colptr = np.empty(b.nrows[1] + 1, dtype=np.int64)
    with pytest.raises(FlexShellError) as e:
        b.ctx.call("fs_batch_matrix_copy", 1, ptr(colptr), None, None)
    assert e.value.code == _abi.FS_ERR_STATE
    # assembled again, the copy gives the same matrices
    Ks2 = b.stiffness(F.SysmatAssemblerSparse())
    for K, K2 in zip(Ks, Ks2):
        assert np.array_equal(K.indptr, K2.indptr) and np.array_equal(K.data, K2.data)
    b.close()

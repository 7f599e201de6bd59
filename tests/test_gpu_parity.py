"""GPU parity of the CUDA library against the oracle, through the C ABI.

Tolerances: the FP64 path must match the oracle within 1e-12 relative
(max-abs difference over max-abs value, per matrix) with an identical
sparsity pattern; the mixed path within 1e-6.
"""
import numpy as np
import pytest
import scipy.linalg as sl

import flexshell as F
from flexshell import _abi
from oracle import oracle as O
import problems as PB
from checks import relmax, same_pattern, same_pattern_modulo_cancellation

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def homog_pair(d, quads, tsf=0):
    et = O.Q4RS if quads else O.T3FF
    P = O.Problem(et, d["xyz"], d["conn"], d["dofnums"], thickness=d["thickness"],
                  material=d["material"], stab_c=d["stab_c"], tsf=tsf)
    P.compute_normals()
    m = d["material"]
    mat = _Mat(m)
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(d["conn"], d["thickness"], mat, stab_fun=d["stab_c"])
    femm.transv_shear_formulation = tsf
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    femm.associategeometry(geom0)
    return P, femm, geom0, dchi


class _Mat:
    """Material given directly by its plane-stress and shear matrices."""

    def __init__(self, m):
        self.m = m

    def massdensity(self):
        return self.m.get("rho", 0.0)


# materials.shell_material_stiffness needs tangentmoduli; route _Mat through it
import flexshell.materials as _materials

_orig = _materials.shell_material_stiffness


def _sms(material):
    if isinstance(material, _Mat):
        return np.asarray(material.m["Dps"]), np.asarray(material.m["Dt"])
    return _orig(material)


_materials.shell_material_stiffness = _sms


@pytest.mark.parametrize("orientation", ["a", "b"])
def test_fv12_gpu_matches_oracle_and_reference(orientation):
    d = PB.fv12(orientation)
    P, femm, geom0, dchi = homog_pair(d, False)
    # normals
    assert np.allclose(femm._normals, P.normals, rtol=0, atol=1e-14)
    assert np.array_equal(femm._normal_valid, P.valid)
    K = femm.stiffness(F.SysmatAssemblerSparseSymm(), geom0, None, None, dchi)
    M = femm.mass(F.SysmatAssemblerSparseSymm(), geom0, dchi)
    Ko = P.assemble_scipy("K", O.DROP_ZEROS)
    Mo = P.assemble_scipy("M", O.DROP_ZEROS)
    assert same_pattern_modulo_cancellation(K, Ko)
    assert same_pattern(M, Mo)
    # the structural pattern (SysmatAssemblerSparse) is bit-exact
    Kk = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    assert same_pattern(Kk, P.assemble_scipy("K", O.KEEP_ZEROS))
    assert relmax(K, Ko) <= FP64_TOL
    assert relmax(M, Mo) <= FP64_TOL
    w = sl.eigh(K.toarray(), M.toarray(), eigvals_only=True)
    fs = np.sqrt(np.abs(w[:14])) / (2 * np.pi)
    np.testing.assert_allclose(fs[6:], np.array(PB.FV12_REF)[6:], rtol=1e-6)
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("n", [4, 8])
def test_scordelis_lo_gpu(quads, n):
    d = PB.scordelis_lo(quads, n)
    P, femm, geom0, dchi = homog_pair(d, quads)
    K = femm.stiffness(F.SysmatAssemblerSparseSymm(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.DROP_ZEROS)
    assert same_pattern_modulo_cancellation(K, Ko)
    assert relmax(K, Ko) <= FP64_TOL
    Kk = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    assert same_pattern(Kk, P.assemble_scipy("K", O.KEEP_ZEROS))
    v = PB.solve_probe(K, d)
    ref = (PB.SLO_Q4_REF if quads else PB.SLO_T3_REF)[PB.SLO_N.index(n)]
    assert abs(v - ref) <= 1e-4 * abs(ref)
    # element matrices, FP64 and mixed
    Ke = femm.element_matrices(geom0, F.FS_FP64)
    Keo = P.element_stiffness()
    assert max(relmax(Ke[e], Keo[e]) for e in range(len(Ke))) <= FP64_TOL
    Km = femm.element_matrices(geom0, F.FS_MIXED)
    assert relmax(Km, Keo) <= MIXED_TOL
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_plate_assemblers_and_mixed(quads):
    xyz, conn, dof, nfree = PB.jittered_plate(12, quads, wavy=0.01, seed=3)
    from flexshell import materials
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    d = dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=0.005,
             material=dict(Dps=Dps, Dt=Dt, rho=7850.0), stab_c=0.1 if quads else 5 / 12 / 1.5)
    P, femm, geom0, dchi = homog_pair(d, quads)
    for asm, mode in ((F.SysmatAssemblerSparse(), O.KEEP_ZEROS),
                      (F.SysmatAssemblerSparseSymm(), O.DROP_ZEROS)):
        K = femm.stiffness(asm, geom0, None, None, dchi)
        Ko = P.assemble_scipy("K", mode)
        if mode == O.KEEP_ZEROS:
            assert same_pattern(K, Ko)
        else:
            assert same_pattern_modulo_cancellation(K, Ko)
        assert relmax(K, Ko) <= FP64_TOL
        Km = femm.stiffness(asm, geom0, None, None, dchi, precision=F.FS_MIXED)
        assert relmax(Km, Ko) <= MIXED_TOL
        M = femm.mass(asm, geom0, dchi)
        Mo = P.assemble_scipy("M", mode)
        assert same_pattern(M, Mo)
        assert relmax(M, Mo) <= FP64_TOL
    # free-free block and diagonal mass
    K = femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS, n=nfree)
    assert same_pattern(K, Ko) and relmax(K, Ko) <= FP64_TOL
    M = femm.mass(F.SysmatAssemblerSparseDiag(), geom0, dchi)
    Mo = P.assemble_scipy("M", O.DIAG)
    assert same_pattern(M, Mo) and relmax(M, Mo) <= FP64_TOL
    # the assembly is deterministic: bitwise identical on a second run
    K1 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    K2 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    assert np.array_equal(K1.data, K2.data)
    femm.close()


def test_t3_average_k_gpu():
    d = PB.scordelis_lo(False, 4)
    P, femm, geom0, dchi = homog_pair(d, False, tsf=1)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert same_pattern(K, Ko) and relmax(K, Ko) <= FP64_TOL
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_composite_gpu(quads):
    plies = PB.cross_ply_groups((30, -45, 60, 0))
    A, B, D, H, md, mi = O.laminate(plies)
    g = F.laminate(plies)
    for name, ref in (("A", A), ("B", B), ("D", D)):
        got = np.array(getattr(g, name)).reshape(3, 3, order="F")
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(A).max()
    c, s = np.cos(0.4), np.sin(0.4)
    cs = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    g.csmat[:] = list(cs.flatten(order="F"))
    t = sum(p["thickness"] for p in plies)
    xyz, conn, dof, nfree = PB.jittered_plate(8, quads, wavy=0.02, seed=7)
    et = O.Q4RSCOMP if quads else O.T3FFCOMP
    stab_c = 0.1 if quads else 5 / 12 / 1.5
    P = O.Problem(et, xyz, conn, dof, groups=[dict(A=A, B=B, D=D, H=H, csmat=cs, thickness=t,
                                                   mass=md, moi=mi)], stab_c=stab_c)
    P.compute_normals()
    cls = F.FEMMShellQ4RSComp if quads else F.FEMMShellT3FFComp
    femm = cls(conn, g, stab_fun=stab_c)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    assert np.allclose(femm._normals, P.normals, atol=1e-14)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert same_pattern(K, Ko) and relmax(K, Ko) <= FP64_TOL
    Km = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=F.FS_MIXED)
    assert relmax(Km, Ko) <= MIXED_TOL
    M = femm.mass(F.SysmatAssemblerSparseSymm(), geom0, dchi)
    Mo = P.assemble_scipy("M", O.DROP_ZEROS)
    assert same_pattern(M, Mo) and relmax(M, Mo) <= FP64_TOL
    femm.close()


def test_errors_are_reported_not_trapped():
    d = PB.scordelis_lo(False, 4)
    femm = F.FEMMShellT3FF(d["conn"], 0.25, _Mat(d["material"]), stab_fun=0.2)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    with pytest.raises(AssertionError):
        femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi)
    bad = d["conn"].copy()
    bad[0, 0] = d["xyz"].shape[0] + 5
    femm2 = F.FEMMShellT3FF(bad, 0.25, _Mat(d["material"]), stab_fun=0.2)
    with pytest.raises(F.FlexShellError) as ei:
        femm2.associategeometry(geom0)
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    femm.close()
    femm2.close()


def test_explicit_steps_match_oracle():
    xyz, conn, dof, nfree = PB.jittered_plate(10, True, seed=2)
    from flexshell import materials
    mat = materials.MatDeforElastIso(200e9, 0.3, 7850.0)
    femm = F.FEMMShellQ4RS(conn, 0.01, mat)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    M = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi)
    K = femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi).tocsr()
    m = M.diagonal()
    w2 = sl.eigh(K.toarray(), np.diag(m), eigvals_only=True)[-1]
    dt = 0.9 * 2 / np.sqrt(w2)
    C = 0.01 * m
    invMC = 1.0 / (m + dt / 2 * C)
    rng = np.random.default_rng(0)
    V0 = rng.normal(0, 1e-3, nfree)
    nsteps = 200
    U, V, A = np.zeros(nfree), V0.copy(), np.zeros(nfree)
    O.cd_steps(K.indptr, K.indices, K.data, invMC, C, dt, nsteps, U, V, A)
    # FP64: double restoring force, so only rounding differs (Kahan state vs plain).
    # Mixed: the restoring force K U is formed in float from float values; K U is
    # a small residual of large terms, so its float rounding shows at ~1e-5 of the
    # velocity after 200 steps (measured 5.4e-5).  Compensated: float values with
    # bf16 residuals, a float-pair U and a compensated float sum (measured 3.5e-9).
    for prec, tol in ((F.FS_FP64, 1e-10), (F.FS_MIXED, 2e-4), (F.FS_MIXED_COMP, 1e-7)):
        ctx = femm.ctx
        import ctypes
        from flexshell._lib import ptr
        invMC_c = np.ascontiguousarray(invMC)
        C_c = np.ascontiguousarray(C)
        ctx.call("fs_explicit_setup", prec, ptr(invMC_c), ptr(C_c), ctypes.c_double(dt))
        z = np.zeros(nfree)
        v0 = V0.copy()
        ctx.call("fs_explicit_set_state", ptr(z), ptr(v0), ptr(z))
        ctx.call("fs_explicit_run", nsteps)
        Ug, Vg, Ag = np.zeros(nfree), np.zeros(nfree), np.zeros(nfree)
        ctx.call("fs_explicit_get_state", ptr(Ug), ptr(Vg), ptr(Ag))
        assert np.abs(Ug - U).max() <= tol * np.abs(U).max()
        assert np.abs(Vg - V).max() <= tol * np.abs(V).max()
    # power iteration for omega_max (the reference's `pwr`) against the dense solution
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    om = ctypes.c_double()
    femm.ctx.call("fs_power_iteration", ptr(np.ascontiguousarray(m)), ctypes.c_int64(2000),
                  ctypes.c_uint64(7), ctypes.byref(om))
    assert abs(om.value - np.sqrt(w2)) <= 1e-3 * np.sqrt(w2)
    femm.close()


def test_explicit_load_matches_oracle():
    # the example's force!(F, t) = g(t) Fmag with the modulated burst of
    # plate_expl_examples.jl:202-209; 150 steps = two captured 64-step graphs
    # plus 22 single steps, then a restart from step 150 with step0
    import ctypes
    from flexshell._lib import ptr
    from flexshell import materials
    xyz, conn, dof, nfree = PB.jittered_plate(10, False, seed=4)
    mat = materials.MatDeforElastIso(200e9, 0.3, 7850.0)
    femm = F.FEMMShellT3FF(conn, 0.01, mat)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    M = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi)
    K = femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi).tocsr()
    m = M.diagonal()
    w2 = sl.eigh(K.toarray(), np.diag(m), eigvals_only=True)[-1]
    dt = 0.9 * 2 / np.sqrt(w2)
    C = 0.02 * m
    invMC = 1.0 / (m + dt / 2 * C)
    rng = np.random.default_rng(5)
    Fmag = rng.normal(0, 1.0, nfree)
    fm, fc = 1 / (120 * dt), 1 / (15 * dt)
    t = np.arange(400) * dt
    mul = np.where(t <= 1 / fm, 0.5 * (1 - np.cos(2 * np.pi * fm * t)) * np.sin(2 * np.pi * fc * t), 0.0)
    nsteps = 150
    U, V = np.zeros(nfree), np.zeros(nfree)
    A = invMC * (mul[0] * Fmag)
    A0 = A.copy()
    O.cd_steps(K.indptr, K.indices, K.data, invMC, C, dt, nsteps, U, V, A, Fmag=Fmag, mul=mul)
    U2, V2, A2 = U.copy(), V.copy(), A.copy()
    O.cd_steps(K.indptr, K.indices, K.data, invMC, C, dt, 50, U2, V2, A2, Fmag=Fmag, mul=mul, step0=nsteps)
    ctx = femm.ctx
    for prec, tol in ((F.FS_FP64, 1e-10), (F.FS_MIXED, 2e-4), (F.FS_MIXED_COMP, 1e-7)):
        ctx.call("fs_explicit_setup", prec, ptr(np.ascontiguousarray(invMC)), ptr(np.ascontiguousarray(C)),
                 ctypes.c_double(dt))
        z = np.zeros(nfree)
        ctx.call("fs_explicit_set_state", ptr(z), ptr(z), ptr(np.ascontiguousarray(A0)))
        ctx.call("fs_explicit_set_load", ptr(Fmag), ptr(mul), mul.shape[0], 0)
        ctx.call("fs_explicit_run", nsteps)
        Ug, Vg, Ag = np.zeros(nfree), np.zeros(nfree), np.zeros(nfree)
        ctx.call("fs_explicit_get_state", ptr(Ug), ptr(Vg), ptr(Ag))
        assert np.abs(Ug - U).max() <= tol * np.abs(U).max()
        assert np.abs(Vg - V).max() <= tol * np.abs(V).max()
        # restart: state and step index given again, then 50 more steps
        ctx.call("fs_explicit_set_state", ptr(Ug), ptr(Vg), ptr(Ag))
        ctx.call("fs_explicit_set_load", ptr(Fmag), ptr(mul), mul.shape[0], nsteps)
        ctx.call("fs_explicit_run", 50)
        ctx.call("fs_explicit_get_state", ptr(Ug), ptr(Vg), ptr(Ag))
        assert np.abs(Ug - U2).max() <= tol * np.abs(U2).max()
        # removing the load: free vibration from the same state
        ctx.call("fs_explicit_set_load", None, None, 0, 0)
        ctx.call("fs_explicit_run", 10)
        U3, V3, A3 = U2.copy(), V2.copy(), A2.copy()
        O.cd_steps(K.indptr, K.indices, K.data, invMC, C, dt, 10, U3, V3, A3)
        ctx.call("fs_explicit_get_state", ptr(Ug), ptr(Vg), ptr(Ag))
        assert np.abs(Ug - U3).max() <= tol * np.abs(U3).max()
    # the Python mirror of _cd_loop! (undamped here: ksi = 0), peeking every 50 steps
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    seen = []
    Uf, Vf, Af = F.cd_loop(femm, m, 0.0, 1.0, np.zeros(nfree), np.zeros(nfree), nsteps * dt, dt, Fmag=Fmag,
                           g=lambda tt: np.interp(tt, t, mul), peek=lambda k, u, v, tt: seen.append(k),
                           peek_every=50)
    U4, V4, A4 = np.zeros(nfree), np.zeros(nfree), invMC * 0.0
    mul4 = np.interp(np.arange(nsteps + 1) * dt, t, mul)
    A4 = (1.0 / m) * (mul4[0] * Fmag)
    O.cd_steps(K.indptr, K.indices, K.data, 1.0 / m, np.zeros(nfree), dt, nsteps, U4, V4, A4, Fmag=Fmag, mul=mul4)
    assert seen == [0, 50, 100, 150]
    assert np.abs(Uf - U4).max() <= 1e-10 * np.abs(U4).max()
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_restoring_force_is_minus_K_U(quads):
    # extension for the shells: F = -K U with U the generalized displacements
    d = PB.scordelis_lo(quads, 6)
    P, femm, geom0, dchi = homog_pair(d, quads)
    rng = np.random.default_rng(4)
    dchi.values = np.asfortranarray(rng.normal(size=dchi.values.shape))
    F = femm.restoringforce(geom0, None, None, dchi)
    n = dchi.nalldofs()
    K = P.assemble_scipy("K", O.KEEP_ZEROS, n=n)
    U = np.zeros(n)
    U[dchi.dofnums.ravel() - 1] = dchi.values.ravel()
    ref = -(K @ U)
    assert np.abs(F - ref).max() <= FP64_TOL * 10 * np.abs(ref).max()
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("asm", [F.SysmatAssemblerSparse, F.SysmatAssemblerSparseSymm])
def test_batch_equals_single_mesh_bitwise(quads, asm):
    # uneven meshes fused into one launch: each mesh's matrix is bitwise the
    # one its own FEMM gives (same element arithmetic, same summation order)
    mat = F.materials.MatDeforElastIso(2.0e11, 0.3, 7850.0)
    meshes, singles = [], []
    for k, n in enumerate([3, 7, 5]):
        xyz, conn, dof, nfree = PB.jittered_plate(n, quads, wavy=0.02, seed=k)
        geom0 = F.NodalField(xyz)
        dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
        dchi.dofnums = np.asfortranarray(dof)
        t = 0.01 * (k + 1)
        meshes.append((geom0, conn, dchi, t))
        cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
        femm = cls(conn, t, mat)
        femm.associategeometry(geom0)
        for prec in (F.FS_FP64, F.FS_MIXED):
            singles.append(femm.stiffness(asm(), geom0, None, None, dchi, precision=prec))
        femm.close()
    b = F.ShellBatch(F.FEMMShellQ4RS if quads else F.FEMMShellT3FF, meshes, mat)
    for j, prec in enumerate((F.FS_FP64, F.FS_MIXED)):
        Ks = b.stiffness(asm(), precision=prec)
        for i, K in enumerate(Ks):
            S = singles[2 * i + j]
            assert same_pattern(K, S)
            assert np.array_equal(K.tocsc().data, S.tocsc().data)
    b.close()


@pytest.mark.parametrize("quads", [False, True])
def test_autotuner_choice_never_changes_the_matrix(quads):
    import ctypes
    mat = F.materials.MatDeforElastIso(2.0e11, 0.3, 7850.0)
    xyz, conn, dof, nfree = PB.jittered_plate(72 if quads else 50, quads, wavy=0.02, seed=1)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(conn, 0.01, mat)
    femm.associategeometry(geom0)
    assert conn.shape[0] >= 4096
    out = (ctypes.c_int32 * 3)()
    for prec in (F.FS_FP64, F.FS_MIXED):
        femm.ctx.call("fs_autotune", 0)
        K0 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=prec)
        femm.ctx.call("fs_tuning", out)
        assert list(out) == [0, 0, 0]
        femm.ctx.call("fs_autotune", 2)
        K1 = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=prec)
        femm.ctx.call("fs_tuning", out)
        assert out[2] == 1 and out[0] > 0 and out[1] in (4, 8, 16)
        assert np.array_equal(K0.data, K1.data) and np.array_equal(K0.indices, K1.indices)
        # a second call reuses the process-wide choice
        femm.ctx.call("fs_autotune", 1)
        femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=prec)
        out2 = (ctypes.c_int32 * 3)()
        femm.ctx.call("fs_tuning", out2)
        assert list(out2) == list(out)
    femm.close()


def test_composite_eigenvalues_mixed_vs_fp64():
    # layered Q4RS plate (scaled-down layered-plate configuration): the 20
    # lowest eigenvalues from the FP64 K match the oracle's to 1e-10, those of
    # the compensated mixed K the FP64 ones to 1e-6
    xyz, conn, dof, nfree, plies = PB.c4_plate(24)
    g = F.laminate(plies)
    femm = F.FEMMShellQ4RSComp(conn, g)
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    asm = F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseSymm(), nfree)
    K64 = femm.stiffness(asm, geom0, None, None, dchi)
    K32 = femm.stiffness(asm, geom0, None, None, dchi, precision=F.FS_MIXED)
    Kc = femm.stiffness(asm, geom0, None, None, dchi, precision=F.FS_MIXED_COMP)
    M = femm.mass(asm, geom0, dchi)
    w64 = PB.lowest_eigenvalues(K64, M)
    w32 = PB.lowest_eigenvalues(K32, M)
    wc = PB.lowest_eigenvalues(Kc, M)
    A, B, D, H, md, mi = O.laminate(plies)
    t = sum(p["thickness"] for p in plies)
    P = O.Problem(O.Q4RSCOMP, xyz, conn, dof, groups=[dict(A=A, B=B, D=D, H=H, csmat=np.eye(3), thickness=t,
                                                            mass=md, moi=mi)])
    P.compute_normals()
    Ko = P.assemble_scipy("K", O.DROP_ZEROS, n=nfree)
    Mo = P.assemble_scipy("M", O.DROP_ZEROS, n=nfree)
    wo = PB.lowest_eigenvalues(Ko, Mo)
    assert w64[0] > 0.0  # no rigid-body mode left
    assert np.abs(w64 - wo).max() <= 1e-10 * np.abs(wo).max()
    # FS_MIXED: the float accumulation of each element's Gram products leaves
    # O(eps |K|) errors in the shear-dominated w-w block of this 1 mm plate,
    # a spurious foundation stiffness that shifts every bending eigenvalue
    # (about 0.07 here, 8e-5 of the lowest); FS_MIXED_COMP accumulates them
    # in compensated sums and keeps the 1e-6 target
    rel = np.abs(w32 - w64) / np.abs(w64)
    assert rel.max() <= 1e-3, rel.max()
    relc = np.abs(wc - w64) / np.abs(w64)
    assert relc.max() <= 1e-6, relc.max()
    assert relmax(Kc, K64) <= MIXED_TOL
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_compensated_mixed_matches_oracle(quads):
    # FS_MIXED_COMP: same pattern, values within the mixed tolerance (curved
    # roof), and on a flat plate, where the element is exactly free of
    # rigid-body stiffness, a rigid translation carries O(eps^2) energy
    # against O(eps) with FS_MIXED
    d = PB.scordelis_lo(quads, 6)
    P, femm, geom0, dchi = homog_pair(d, quads)
    Kc = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=F.FS_MIXED_COMP)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert same_pattern(Kc, Ko) and relmax(Kc, Ko) <= MIXED_TOL
    femm.close()
    xyz, conn, dof, nfree = PB.jittered_plate(6, quads, seed=3)
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(conn, 0.001, F.materials.MatDeforElastIso(2.0e11, 0.3, 7850.0))
    geom0 = F.NodalField(xyz)
    femm.associategeometry(geom0)
    E64 = femm.element_matrices(geom0, precision=F.FS_FP64)
    Ec = femm.element_matrices(geom0, precision=F.FS_MIXED_COMP)
    Em = femm.element_matrices(geom0, precision=F.FS_MIXED)
    u = np.zeros(E64.shape[1]); u[0::6] = 1.0          # rigid x translation
    e64 = np.abs(np.einsum("i,eij,j->e", u, E64, u)).max()
    ec = np.abs(np.einsum("i,eij,j->e", u, Ec, u)).max()
    em = np.abs(np.einsum("i,eij,j->e", u, Em, u)).max()
    scale = np.abs(E64).max()
    assert e64 <= 1e-13 * scale
    assert ec <= 1e-12 * scale and ec <= em
    femm.close()


@pytest.mark.parametrize("precision", [F.FS_FP64, F.FS_MIXED])
def test_two_phase_copy_equals_stiffness_and_copy(precision):
    import ctypes
    from flexshell._lib import ptr
    d = PB.scordelis_lo(True, 6)
    P, femm, geom0, dchi = homog_pair(d, True)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, dchi, precision=precision)
    n = dchi.nalldofs()
    nnz = ctypes.c_int64()
    femm.ctx.call("fs_pattern", n, ctypes.byref(nnz))
    assert nnz.value == K.nnz
    colptr = np.empty(n + 1, dtype=np.int64)
    rowval = np.empty(nnz.value, dtype=np.int64)
    nzval = np.empty(nnz.value)
    femm.ctx.call("fs_stiffness_copy", precision, n, ptr(colptr), ptr(rowval), ptr(nzval))
    assert np.array_equal(colptr - 1, K.indptr) and np.array_equal(rowval - 1, K.indices)
    assert np.array_equal(nzval, K.data)
    femm.close()


def test_explicit_smooth_field_error_by_mode():
    """The explicit configuration at 48 x 48 (Q4RS, t = 0.01, steel, simply
    supported, V0 = 1e-3 sin(pi x) sin(pi y) plus seeded noise, 0.9 dt_crit,
    1,500 steps): final displacements of the mixed and compensated steps
    against the FP64 step.  A smooth field is where K U cancels most: the
    plain mixed step is off by 1e-5..1e-4 of max |U| here, the compensated
    one (float values with bf16 residuals, float-pair U, compensated float
    sum) by 1e-9..1e-8 (9.9e-9 at 128 x 128 after 2,500 steps, 5.5e-7 at
    512 x 512 after 10,000)."""
    import ctypes
    from flexshell import materials, mesh
    from flexshell._lib import ptr
    n, nsteps = 48, 1500
    xyz, conn = mesh.jittered_plate_q(n, 1.0, 0.0, 0, None)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    x, y = xyz[:, 0], xyz[:, 1]
    fixed[(x < 1e-12) | (x > 1 - 1e-12) | (y < 1e-12) | (y > 1 - 1e-12), 2] = True
    dof, nfree = mesh.numberdofs(fixed)
    femm = F.FEMMShellQ4RS(conn, 0.01, materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    geom0 = F.NodalField(xyz)
    dchi = F.NodalField(np.zeros((xyz.shape[0], 6)))
    dchi.dofnums = np.asfortranarray(dof)
    femm.associategeometry(geom0)
    m = femm.mass(F.SysmatAssemblerFFBlock(F.SysmatAssemblerSparseDiag(), nfree), geom0, dchi).diagonal()
    femm.stiffness(F.SysmatAssemblerFFBlock(nfree), geom0, None, None, dchi)
    om = ctypes.c_double()
    femm.ctx.call("fs_power_iteration", ptr(np.ascontiguousarray(m)), ctypes.c_int64(300), ctypes.c_uint64(1),
                  ctypes.byref(om))
    dt = 0.9 * 2 / om.value
    rng = np.random.Generator(np.random.PCG64(5))
    V0 = np.zeros(nfree)
    wd = dof[:, 2]
    fw = wd <= nfree
    V0[wd[fw] - 1] = 1e-3 * np.sin(np.pi * x[fw]) * np.sin(np.pi * y[fw]) + rng.normal(0, 1e-5, fw.sum())
    invMC = np.ascontiguousarray(1.0 / m)
    C = np.zeros(nfree)
    finals = {}
    for prec in (F.FS_FP64, F.FS_MIXED, F.FS_MIXED_COMP):
        femm.ctx.call("fs_explicit_setup", prec, ptr(invMC), ptr(C), ctypes.c_double(dt))
        z = np.zeros(nfree)
        femm.ctx.call("fs_explicit_set_state", ptr(z), ptr(np.ascontiguousarray(V0)), ptr(z))
        femm.ctx.call("fs_explicit_run", ctypes.c_int64(nsteps))
        U = np.zeros(nfree)
        femm.ctx.call("fs_explicit_get_state", ptr(U), None, None)
        finals[prec] = U
    ref = finals[F.FS_FP64]
    err = {p: np.abs(finals[p] - ref).max() / np.abs(ref).max() for p in (F.FS_MIXED, F.FS_MIXED_COMP)}
    assert err[F.FS_MIXED] <= 1e-3, err
    assert err[F.FS_MIXED_COMP] <= 1e-7, err
    assert err[F.FS_MIXED_COMP] <= err[F.FS_MIXED] / 100, err
    femm.close()

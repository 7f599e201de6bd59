"""GPU parity of the distributed loads (fs_distribloads,
fs_integration_points: FinEtools distribloads on the shell element sets, as
test/test_shell_statics.jl:84-86 and plate_expl_examples.jl:196-199 call it,
and on the L2 edges of their boundary, test/test_shell_statics.jl:212-215)
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


def test_line_loads_match_oracle():
    # the boundary curves of a T3 and a Q4 mesh: every GaussRule(1, order), m,
    # uniform, per-element and per-point force, and a callable
    for quads in (False, True):
        d, geom0, dchi = _setup(quads)
        edges = F.mesh.meshboundary(d["conn"])
        n = dchi.nalldofs()
        q = np.array([0.5, -0.25, -90.0, 0.01, -0.02, 0.03])
        for order in (1, 2, 3):
            lfemm = F.FEMMBase(F.IntegDomain(edges, F.GaussRule(1, order)))
            for m in (1, 2, 3):
                Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(q), m)
                Fo = O.distribloads(d["xyz"], edges, d["dofnums"], order, m, q, n)
                assert Fg.shape == (n,) and _rel(Fg, Fo) <= 1e-12
            pts = lfemm.integration_points(geom0)
            po = O.integration_points(d["xyz"], edges, order)
            assert pts.shape == (edges.shape[0] * order, 9)
            assert np.abs(pts - po).max() <= 1e-12 * np.abs(po).max()
            assert np.all(pts[:, 6:9] == 0.0)
            fp = np.random.default_rng(order).normal(size=(pts.shape[0], 6))
            out = np.zeros(n)
            lfemm.ctx.call("fs_distribloads", order, 1, ptr(fp), fp.shape[0], n, ptr(out))
            assert _rel(out, O.distribloads(d["xyz"], edges, d["dofnums"], order, 1, fp, n)) <= 1e-12
            fe = fp[: edges.shape[0]]
            lfemm.ctx.call("fs_distribloads", order, 2, ptr(fe), fe.shape[0], n, ptr(out))
            assert _rel(out, O.distribloads(d["xyz"], edges, d["dofnums"], order, 2, fe, n)) <= 1e-12

            def computetrac(forceout, XYZ, tangents, feid, qpid):
                assert tangents.shape == (3, 1)
                forceout[:] = 0.0
                forceout[1] = XYZ[0, 0] * np.linalg.norm(tangents)
                return forceout

            Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(float, 6, computetrac), 1)
            fpts = np.zeros((po.shape[0], 6))
            fpts[:, 1] = po[:, 0] * np.linalg.norm(po[:, 3:6], axis=1)
            assert _rel(Fg, O.distribloads(d["xyz"], edges, d["dofnums"], order, 1, fpts, n)) <= 1e-12
            with pytest.raises(FlexShellError) as ei:
                lfemm.ctx.call("fs_distribloads", 4, 1, ptr(q), 1, n, ptr(out))
            assert ei.value.code == _abi.FS_ERR_BAD_INPUT
            lfemm.close()


@pytest.mark.parametrize("k", range(4))
def test_raasch_hook_on_gpu(k):
    # test/test_shell_statics.jl:229-236 (rtol 1e-4): the reference's Abaqus
    # meshes, stiffness and tip-edge load both from the GPU
    d = PB.raasch_hook(k)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    mat = F.materials.MatDeforElastIso(3300.0, 0.35)
    femm = F.FEMMShellT3FF(d["conn"], d["thickness"], mat, stab_fun=d["stab_c"])
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    lfemm = F.FEMMBase(F.IntegDomain(d["edges"], F.GaussRule(1, 2)))
    Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(d["traction"]), 3)
    Fo = O.distribloads(d["xyz"], d["edges"], d["dofnums"], 2, 3, d["traction"], dchi.nalldofs())
    assert _rel(Fg, Fo) <= 1e-12
    v = PB.tip_deflection_percent(K, Fg, d)
    assert abs(v - PB.RAASCH_REF[k]) <= 1e-4 * abs(PB.RAASCH_REF[k])
    assert abs(v - PB.RAASCH_REF[k]) <= 1e-9 * abs(PB.RAASCH_REF[k])
    femm.close()
    lfemm.close()


@pytest.mark.parametrize("quads", [False, True])
def test_barbero_layered_plate_on_gpu(quads):
    # test/test_composite_shell_statics.jl:14-97 and
    # test/test_composite_shell_statics_q4rs.jl:14-97 (`≈`, rtol sqrt(eps)):
    # [0/90] plate, layered stiffness and the in-plane edge loads over the
    # boundary's L2 elements, all from the GPU
    import scipy.sparse.linalg as spl
    d = PB.barbero_plate(quads)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    g = F.laminate(d["plies"])
    femm = (F.FEMMShellQ4RSComp if quads else F.FEMMShellT3FFComp)(d["conn"], g)
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    Fg = np.zeros(dchi.nalldofs())
    for edges, f in d["edge_loads"]:
        lfemm = F.FEMMBase(F.IntegDomain(edges, F.GaussRule(1, 2)))
        Fg += F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(f), 1)
        lfemm.close()
    assert _rel(Fg, d["F"]) <= 1e-12
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), Fg[:nf])
    dz = d["dofnums"][:, 2]
    uz = np.where(dz <= nf, u[np.minimum(dz, nf) - 1], 0.0)
    ref = PB.BARBERO_Q4_UZMAX_MM if quads else PB.BARBERO_T3_UZMAX_MM
    assert abs(uz.max() / 1e-3 - ref) <= 1.5e-8 * ref
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("example", ["3.1x10", "3.3", "r+", "r-", "rot+", "rot-", "p0/90", "p-45/45"])
def test_barbero_examples_on_gpu(quads, example):
    # test/test_composite_shell_statics.jl:117-200, :234-323, :683-753,
    # :774-844, :870-954, :978-1075 and the Q4RS file's same tests (`≈`, rtol
    # sqrt(eps)): twenty [0/90] plies, the [+45/-45/0/0/-45/+45] layup pulled in
    # x, [90/0] pulled and pushed, the same plate turned into the y-z plane
    # with a rotated layup csys, or [0/90] and [-45/+45] under pressure;
    # stiffness and loads from the GPU
    d = PB.barbero_example(quads, example)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    g = F.laminate(d["plies"])
    g.csmat[:] = list(np.asarray(d["csmat"]).flatten(order="F"))
    femm = (F.FEMMShellQ4RSComp if quads else F.FEMMShellT3FFComp)(d["conn"], g)
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    Fg = np.zeros(dchi.nalldofs())
    for edges, f in d["edge_loads"]:
        lfemm = F.FEMMBase(F.IntegDomain(edges, F.GaussRule(1, 2)))
        Fg += F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(f), 1)
        lfemm.close()
    if d["surface_load"] is not None:
        rule, f = d["surface_load"]
        lfemm = F.FEMMBase(F.IntegDomain(d["conn"], F.GaussRule(2, rule) if quads else F.TriRule(rule)))
        Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(f), 2)
        lfemm.close()
    v = PB.max_displacement_mm(K, Fg, d)
    assert abs(v - d["ref"]) <= 1.5e-8 * abs(d["ref"])
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("example", ["sacco", "sandwich"])
def test_sacco_and_sandwich_plates_on_gpu(quads, example):
    # test/test_composite_shell_statics.jl:1099-1183, :1210-1282 and the Q4RS
    # file's same tests (`≈`, rtol sqrt(eps)): stiffness and pressure from the GPU
    d = PB.sacco_and_sandwich(quads, example)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    femm = (F.FEMMShellQ4RSComp if quads else F.FEMMShellT3FFComp)(d["conn"], F.laminate(d["plies"]))
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    rule, f = d["surface_load"]
    lfemm = F.FEMMBase(F.IntegDomain(d["conn"], F.GaussRule(2, rule) if quads else F.TriRule(rule)))
    Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(f), 2)
    lfemm.close()
    for v, ref in PB.extreme_displacements(K, Fg, d):
        assert abs(v - ref) <= 1.5e-8 * abs(ref)
    femm.close()


def test_le5_z_cantilever_on_gpu():
    # test/test_shell_statics.jl:525-531 (`≈`, rtol sqrt(eps)): T3FF stiffness
    # of the reference's Z-section mesh from the GPU
    d = PB.le5_cantilever()
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    femm = F.FEMMShellT3FF(d["conn"], d["thickness"], F.materials.MatDeforElastIso(210e9, 0.3),
                           stab_fun=d["stab_c"])
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    for v, ref in zip(PB.w_extremes(K, d["F"], d), PB.LE5_REF):
        assert abs(v - ref) <= 1.5e-8 * abs(ref)
    femm.close()


def test_barrel_vault_resultant_fields_on_gpu():
    # test/test_shell_statics.jl:578-727 (rtol 0.01): stiffness, load,
    # resultants at the integration points in the cylindrical output csys from
    # the GPU; fieldfromintegpoints' inverse-distance node values on the host
    d = PB.barrel_vault()
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    dchi.nfreedofs = d["nfree"]
    femm = F.FEMMShellT3FF(d["conn"], d["thickness"], F.materials.MatDeforElastIso(3.0e6, 0.0),
                           stab_fun=d["stab_c"])
    femm.drilling_stiffness_scale = d["drill_scale"]
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    lfemm = F.FEMMBase(F.IntegDomain(d["conn"], F.TriRule(3)))
    Fg = F.distribloads(lfemm, geom0, dchi, F.ForceIntensity(d["load"]), 3)
    lfemm.close()
    U = PB.nodal_displacements(K, Fg, d)
    for name, refs in PB.VAULT_REF.items():
        for nc, (rmin, rmax) in enumerate(refs):
            f = femm.fieldfromintegpoints(geom0, U, name, nc + 1, outputcsys=d["ocsys"])
            assert abs(f.min() - rmin) <= 0.01 * abs(rmin) and abs(f.max() - rmax) <= 0.01 * abs(rmax)
    femm.close()


@pytest.mark.parametrize("layered", [False, True])
def test_petyt_plate_frequencies_on_gpu(layered):
    # test/test_composite_shell_dynamics.jl:93-104, :192-203 (|f - f_ref| <
    # 1e-3 |f|; measured 2e-9 per frequency on the oracle): stiffness and
    # lumped mass from the GPU
    d = PB.petyt_plate()
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    if layered:
        femm = F.FEMMShellT3FFComp(d["conn"], F.laminate(d["plies"]))
    else:
        femm = F.FEMMShellT3FF(d["conn"], d["thickness"], F.materials.MatDeforElastIso(d["E"], d["nu"], d["rho"]))
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    M = femm.mass(geom0, dchi)
    fs = PB.lowest_frequencies(K, M, d["nfree"], 8)
    assert np.linalg.norm(fs - PB.PETYT_REF) < 1e-3 * np.linalg.norm(fs)
    np.testing.assert_allclose(fs, PB.PETYT_REF, rtol=1e-8)
    femm.close()


@pytest.mark.parametrize("case", range(4))
def test_nayak_plate_frequencies_on_gpu(case):
    # test/test_composite_shell_dynamics.jl:432-443, 457-460 (|f - f_ref| <
    # 1e-13 on the nondimensional frequencies): layered stiffness and lumped
    # mass from the GPU for the four layups and layup csys axes
    nplies, axes = PB.NAYAK_CASES[case]
    d = PB.nayak_plate(nplies, axes)
    geom0 = F.NodalField(d["xyz"])
    dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
    dchi.dofnums = np.asfortranarray(d["dofnums"])
    g = F.laminate(d["plies"])
    g.csmat[:] = list(np.asarray(d["csmat"]).flatten(order="F"))
    femm = F.FEMMShellT3FFComp(d["conn"], g)
    femm.associategeometry(geom0)
    K = femm.stiffness(geom0, None, None, dchi)
    M = femm.mass(geom0, dchi)
    fs = PB.lowest_frequencies(K, M, d["nfree"], 9)
    assert np.linalg.norm(np.array(PB.NAYAK_REF) - d["scale"] * fs) < 1e-13
    femm.close()


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("k", range(4))
def test_twisted_beam_on_gpu(k, quads):
    # test/test_shell_statics.jl:362-400 and test/test_q4rs_shell_statics.jl:
    # 358-400 (rtol 1e-3): T3FF and Q4RS stiffness of the twisted beams from
    # the GPU, and its tip value against the oracle's (same solver).  The
    # thin beams (k = 2, 3) are ill-conditioned: a relative perturbation of
    # 2.2e-16 of the oracle's own K moves their tip value by up to 2.1e-5 of
    # the reference (1.3e-9 for k = 0, 1), so the bound against the oracle
    # is 6e-5 there and 1e-8 for the thick beams.
    tol = 6e-5 if k >= 2 else 1e-8
    for j in range(4):
        d = PB.twisted_beam(k, j, quads)
        geom0 = F.NodalField(d["xyz"])
        dchi = F.NodalField(np.zeros((d["xyz"].shape[0], 6)))
        dchi.dofnums = np.asfortranarray(d["dofnums"])
        femm = (F.FEMMShellQ4RS if quads else F.FEMMShellT3FF)(
            d["conn"], d["thickness"], F.materials.MatDeforElastIso(d["E"], d["nu"]), stab_fun=d["stab_c"])
        femm.associategeometry(geom0)
        v = PB.twisted_tip_percent(femm.stiffness(geom0, None, None, dchi), d)
        P = O.Problem(O.Q4RS if quads else O.T3FF, d["xyz"], d["conn"], d["dofnums"], thickness=d["thickness"],
                      material=d["material"], stab_c=d["stab_c"])
        P.compute_normals()
        vo = PB.twisted_tip_percent(P.assemble_scipy("K", O.KEEP_ZEROS).tocsr(), d)
        assert abs(v - d["ref"]) <= 1e-3 * abs(d["ref"])
        assert abs(v - vo) <= tol * abs(d["ref"])
        femm.close()

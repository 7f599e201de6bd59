"""Problem builders shared by the oracle pins and the GPU parity tests.

Each builder restates the set-up of a reference test (mesh, material,
boundary conditions) using the FinEtools-equivalent helpers of
``flexshell.mesh``.
"""
import numpy as np

from flexshell import mesh, materials

PHI40 = 40 / 360 * 2 * np.pi


def fv12(orientation="a", n=8):
    """NAFEMS FV12 free plate, test/test_shell_dynamics.jl:27-66."""
    E, nu, rho, t, L = 200e9, 0.3, 8000.0, 0.05, 10.0
    xy, conn = mesh.T3block(L, L, n, n, orientation)
    xy[:, 0] -= L / 2
    xy[:, 1] -= L / 2
    xyz = mesh.xyz3(xy)
    mat = materials.MatDeforElastIso(E, nu, rho)
    Dps, Dt = materials.shell_material_stiffness(mat)
    dof, nfree = mesh.numberdofs(np.zeros((xyz.shape[0], 6), bool))
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=rho), stab_c=0.2)


# test/test_shell_dynamics.jl:113-128
FV12_REF = [0.0, 0.0, 2.604869127850317e-7, 4.698288861559094e-6, 6.749716652051837e-6,
            9.829373450823236e-6, 1.572130183778014, 2.2424585076387427, 2.8079394352847316,
            3.883763676656034, 4.039123204140305, 6.787320617260535, 6.920636670319986,
            7.127888889722697]

# test/test_shell_statics.jl:97-104 and test/test_q4rs_shell_statics.jl:95-101
SLO_N = [4, 8, 10, 12, 16, 24]
SLO_T3_REF = [66.54771615057949, 85.54615143134853, 89.85075281481419, 92.50616661644985,
              95.40469210310079, 97.65376880486126]
SLO_Q4_REF = [97.88098976068304, 98.766679964194, 99.1305903792941, 99.33597700449404,
              99.52904556664862, 99.63694998474682]


def scordelis_lo(quads, n):
    """Scordelis-Lo roof, test/test_shell_statics.jl:14-90 (T3) and
    test/test_q4rs_shell_statics.jl:14-88 (Q4)."""
    E, nu, t, R, L = 4.32e8, 0.0, 0.25, 25.0, 50.0
    tol = R / n / 1000
    if quads:
        xy, conn = mesh.Q4block(PHI40, L / 2, n, n)
    else:
        xy, conn = mesh.T3block(PHI40, L / 2, n, n)
    a, y = xy[:, 0].copy(), xy[:, 1].copy()
    xyz = np.stack([R * np.sin(a), y, R * (np.cos(a) - 1)], 1)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    inf = np.inf
    l1 = mesh.selectnode(xyz, [-inf, inf, 0, 0, -inf, inf], tol) - 1
    for i in [1, 3, 5]:
        fixed[l1, i - 1] = True
    l1 = mesh.selectnode(xyz, [-inf, inf, L / 2, L / 2, -inf, inf], tol) - 1
    for i in [2, 4, 6]:
        fixed[l1, i - 1] = True
    l1 = mesh.selectnode(xyz, [0, 0, -inf, inf, -inf, inf], tol) - 1
    for i in [1, 5, 6]:
        fixed[l1, i - 1] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, nu))
    nl = mesh.selectnode(xyz, [np.sin(PHI40) * 25] * 2 + [L / 2, L / 2, -inf, inf], tol)[0] - 1
    F = surface_load(xyz, conn, dof, -90.0)
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=0.0), stab_c=0.2, F=F, probe=nl)


# test/test_shell_statics.jl:229-236: tip deflection in percent of 5.02
RAASCH_MESHES = ["1x9", "3x18", "5x36", "10x72"]
RAASCH_REF = [91.7059961843231, 95.9355786538892, 97.19276899988246, 98.38896641657374]


def raasch_hook(k):
    """Raasch hook, test/test_shell_statics.jl:143-227: the reference's Abaqus
    meshes (tests/golden/raasch_hook.npz), Q4toT3, clamped at x = 0, a shear
    traction of 0.05 in z on the tip edge (meshboundary, GaussRule(1, 2),
    distribloads m = 3).  Returns the problem and the tip edges."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "raasch_hook.npz"))
    m = RAASCH_MESHES[k]
    xyz, conn = g["xyz_" + m], mesh.Q4toT3(g["conn_" + m])
    E, nu, t = 3300.0, 0.35, 2.0
    tol = t / 2
    inf = np.inf
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[mesh.selectnode(xyz, [0, 0, -inf, inf, -inf, inf], tol) - 1, :] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, nu))
    bfes = mesh.meshboundary(conn)
    edges = bfes[mesh.selectelem(xyz, bfes, [97.9615, 97.9615, -16, -16, 0, 20], tol)]
    probe = mesh.selectnode(xyz, [97.9615, 97.9615, -16, -16, 0, 0], tol)[0] - 1
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=0.0), stab_c=0.2, probe=probe,
                edges=edges, traction=np.array([0, 0, 0.05, 0, 0, 0.0]))


# test/test_shell_statics.jl:530-531 (`≈`, rtol sqrt(eps)): min and max w
LE5_REF = (-0.01568028415401719, 0.015401663810490641)


def le5_cantilever():
    """LE5 Z-section cantilever, test/test_shell_statics.jl:441-531: the
    reference's Abaqus triangles (tests/golden/raasch_hook.npz), translations
    clamped at x = 0, opposite point forces of 0.6 MN in z at (10, 1, 0) and
    (10, -1, 0) (FESetP1 with PointRule: the force itself at the node)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "raasch_hook.npz"))
    xyz, conn = g["xyz_le5"], g["conn_le5"]
    tol = 0.1 / 1000
    inf = np.inf
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[mesh.selectnode(xyz, [0, 0, -inf, inf, -inf, inf], tol) - 1, 0:3] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(210e9, 0.3))
    F = np.zeros(int(dof.max()))
    for y, fz in ((1.0, 0.6e6), (-1.0, -0.6e6)):
        nl = mesh.selectnode(xyz, [10, 10, y, y, 0, 0], tol) - 1
        assert nl.size == 1
        F[dof[nl[0], 2] - 1] += fz
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=0.1,
                material=dict(Dps=Dps, Dt=Dt, rho=0.0), stab_c=0.2, F=F)


# test/test_shell_statics.jl:690-727: (min, max) of the nodal fields of the
# moments, membrane forces and shears (rtol 0.01)
VAULT_REF = {"moment": [(-1520.6449167366522, 14.067403309095397), (-73.8262145426215, 425.93651541819503),
                        (-0.005341121492547284, 953.0929383629322)],
             "membrane": [(-306.83173146926623, 309.5860993742647), (-1011.4832977998705, 2167.0403478574167),
                          (-687.3500043290137, 69.38703021678862)],
             "shear": [(-13.784764125688811, 21.165312065421237), (-7.4216963152916255, 25.679801383392967)]}


def barrel_vault():
    """Irregular barrel vault, test/test_shell_statics.jl:578-727: the
    reference's Abaqus triangles (tests/golden/raasch_hook.npz) with coincident
    nodes merged (mergenodes, t/10), E = 3e6, nu = 0, t = 3, stab 0.2,
    drilling scale 0.1, gravity-like load -0.625 in x (TriRule(3), m = 3).
    Also returns the cylindrical output csys of the resultants."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "raasch_hook.npz"))
    t, R, L = 3.0, 300.0, 600.0
    xyz, conn = mesh.mergenodes(g["xyz_vault"], g["conn_vault"], t / 10)
    tol = t / 20
    inf = np.inf
    fixed = np.zeros((xyz.shape[0], 6), bool)
    for box, comps in (([-inf, inf, -inf, inf, 0, 0], [0, 1]), ([-inf, inf, -inf, inf, L / 2, L / 2], [2, 3, 4]),
                       ([-inf, inf, 0, 0, -inf, inf], [1, 3, 5])):
        fixed[np.ix_(mesh.selectnode(xyz, box, tol) - 1, comps)] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(3.0e6, 0.0))

    def cylindrical(XYZ, tangents, feid, qpid):
        r = -np.asarray(XYZ, dtype=np.float64).ravel().copy()
        r[2] = 0.0
        e3 = r / np.linalg.norm(r)
        e2 = np.array([0.0, 0.0, 1.0])
        return np.column_stack([np.cross(e2, e3), e2, e3])

    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=0.0), stab_c=0.2, drill_scale=0.1,
                load=np.array([-0.625, 0, 0, 0, 0, 0.0]), ocsys=cylindrical)


def nodal_displacements(K, F, d):
    """K_ff u = F_f scattered back to the (nnodes, 6) nodal values."""
    import scipy.sparse.linalg as spl
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), F[:nf])
    dof = d["dofnums"]
    return np.where(dof <= nf, u[np.minimum(dof, nf) - 1], 0.0)


def inverse_distance_field(xyz, conn, vals):
    """Nodal field of one value per T3 element (its centroid), FinEtools'
    inverse-distance node values (weights 1/|x_node - x_point|^2)."""
    loc = xyz[conn - 1].mean(axis=1)
    num = np.zeros(xyz.shape[0])
    den = np.zeros(xyz.shape[0])
    for e in range(conn.shape[0]):
        for a in conn[e] - 1:
            w = 1.0 / ((xyz[a] - loc[e]) ** 2).sum()
            num[a] += w * vals[e]
            den[a] += w
    return num / den


# test/test_composite_shell_dynamics.jl:93-104 and :192-203 (norm of the
# difference below 1e-3 of the norm)
PETYT_REF = [21.822774909379287, 54.52203720717488, 54.60475772077202, 86.5480437899711,
             108.65349048567792, 108.78050954575491, 138.29506871044424, 140.89370172063866]


def petyt_plate():
    """Simply supported square plate of Petyt 9.2,
    test/test_composite_shell_dynamics.jl:19-104 (T3FF) and :108-203 (T3FFComp,
    four isotropic plies at +-45 degrees): 1 m, 8 x 8 T3, E = 1 GPa,
    nu = 0.396, rho = 2, t = 1 mm, translations fixed on the boundary."""
    E, nu, rho, t = 1.0e9, 0.396, 2.0, 1.0e-3
    xy, conn = mesh.T3block(1.0, 1.0, 8, 8)
    xyz = mesh.xyz3(xy)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[np.unique(mesh.meshboundary(conn)) - 1, 0:3] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, nu, rho))
    plies = [dict(Dps=Dps, Dts=Dt, thickness=t / 4, angle=a, rho=rho) for a in (45.0, -45.0, 45.0, -45.0)]
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=rho), plies=plies, E=E, nu=nu, rho=rho)


# test/test_composite_shell_dynamics.jl:432-443 (norm of the difference below 1e-13)
NAYAK_REF = [0.04571652264814249, 0.10096323319412286, 0.11467782865238098, 0.16264669289730896,
             0.18683613787902217, 0.20655080934826295, 0.23954509827380233, 0.2476225295798577,
             0.2718218525817157]
NAYAK_CASES = [(10, (1, 2, 3)), (3, (2, -1, 3)), (5, (-1, -2, 3)), (4, (-2, 1, 3))]


def cartesian_csys(axes):
    """CompositeLayupModule.cartesian_csys: column j is sign(axes[j]) times
    the unit vector of axis |axes[j]| (src/CompositeLayupModule.jl:26-40)."""
    cs = np.zeros((3, 3))
    for j, a in enumerate(axes):
        cs[abs(a) - 1, j] = np.sign(a)
    return cs


def nayak_plate(nplies, axes):
    """Nayak 4.3 orthotropic plate, test/test_composite_shell_dynamics.jl:353-443:
    100 mm, 9 x 9 T3, t = ax/10 in nplies equal 0-degree plies, layup csys
    cartesian_csys(axes), translations fixed on the boundary."""
    from flexshell import materials
    ax = 0.1
    rho = 1500.0
    mat = materials.lamina_material(rho, 143.52e9, 75.38e9, 0.44, 42.03e9, 25.56e9, 42.65e9)
    Dps, Dts = materials.shell_material_stiffness(mat)
    t = ax / 10
    plies = [dict(Dps=Dps, Dts=Dts, thickness=t / nplies, angle=0.0, rho=rho) for _ in range(nplies)]
    xy, conn = mesh.T3block(ax, ax, 9, 9)
    xyz = mesh.xyz3(xy)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[np.unique(mesh.meshboundary(conn)) - 1, 0:3] = True
    dof, nfree = mesh.numberdofs(fixed)
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t, plies=plies,
                csmat=cartesian_csys(axes), scale=t * np.sqrt(rho / 159.85e9) * 2 * np.pi)


def lowest_frequencies(K, M, nfree, n):
    """The n lowest natural frequencies (Hz) of the free-free blocks."""
    import scipy.linalg as sl
    Kf = K[:nfree, :nfree].toarray()
    Mf = M[:nfree, :nfree].toarray()
    w = sl.eigh(Kf, Mf, eigvals_only=True, subset_by_index=[0, n - 1])
    return np.sqrt(np.abs(w)) / (2 * np.pi)


# test/test_shell_statics.jl:287-291, 364-381 (rtol 1e-3): tip deflection
# in percent of uex for n = 2, 4, 8, 16 (2n x n mesh) per parameter set
TWIST_PARAMS = [(0.32, 1.0, 2, 0.001753248285256), (0.32, 1.0, 3, 0.005424534868469),
                (0.0032, 1.0e-6, 2, 0.001294), (0.0032, 1.0e-6, 3, 0.005256)]
TWIST_N = [2, 4, 8, 16]
TWIST_REF = [39.709921740907355, 68.87306876326497, 86.01944734315117, 95.04101960524827,
             53.10262177376127, 83.8593790803426, 94.91359387874728, 98.21549248655576,
             48.16757753755567, 79.43420077873479, 92.54464819755955, 96.85008269135751,
             50.577029703967334, 80.34160167730624, 92.48675665271801, 96.7096641005938]


# test/test_q4rs_shell_statics.jl:360-377, the same sets on Q4block meshes
TWIST_Q4_REF = [57.52004303100694, 82.57318302555431, 94.20131995162048, 98.37454367262973,
                76.28227868667001, 93.90901921611645, 98.28145099724978, 99.43562910255783,
                68.51008267652144, 90.66189189880987, 97.4223162100464, 99.27913153086936,
                76.09971224380796, 93.00031411228612, 97.58071557550575, 99.2319932521005]


def twisted_beam(k, j, quads=False):
    """Twisted beam, test/test_shell_statics.jl:294-360 (T3FF, T3block 'a')
    and test/test_q4rs_shell_statics.jl:288-355 (Q4RS, Q4block, stab
    t^2/(t^2 + 0.05 h^2)): parameter set k, mesh 2n x n with n = TWIST_N[j],
    twisted by 90 degrees along its length, clamped at x = 0, a point force at
    the tip centre."""
    t, force, direction, uex = TWIST_PARAMS[k]
    n = TWIST_N[j]
    E, nu, W, L = 0.29e8, 0.22, 1.1, 12.0
    tol = W / n / 100
    xy, conn = mesh.Q4block(L, W, 2 * n, n) if quads else mesh.T3block(L, W, 2 * n, n, "a")
    xyz = mesh.xyz3(xy)
    a = xyz[:, 0] / L * (np.pi / 2)
    y = xyz[:, 1] - W / 2
    z = xyz[:, 2].copy()
    xyz = np.column_stack([xyz[:, 0], y * np.cos(a) - z * np.sin(a), y * np.sin(a) + z * np.cos(a)])
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[mesh.selectnode(xyz, [0, 0, -np.inf, np.inf, -np.inf, np.inf], tol) - 1, :] = True
    dof, nfree = mesh.numberdofs(fixed)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, nu))
    nl = mesh.selectnode(xyz, [L, L, 0, 0, 0, 0], tol) - 1
    assert nl.size == 1
    F = np.zeros(int(dof.max()))
    F[dof[nl[0], direction - 1] - 1] = force
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, thickness=t,
                material=dict(Dps=Dps, Dt=Dt, rho=0.0), stab_c=0.05 if quads else 5 / 12 / 1.5, F=F,
                probe=(nl[0], direction - 1), uex=uex, E=E, nu=nu,
                ref=(TWIST_Q4_REF if quads else TWIST_REF)[4 * k + j])


def twisted_tip_percent(K, d):
    import scipy.sparse.linalg as spl
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), d["F"][:nf])
    node, comp = d["probe"]
    return u[d["dofnums"][node, comp] - 1] / d["uex"] * 100


def w_extremes(K, F, d):
    """K_ff u = F_f; (min, max) of the nodal z displacements."""
    import scipy.sparse.linalg as spl
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), F[:nf])
    dz = d["dofnums"][:, 2]
    w = np.where(dz <= nf, u[np.minimum(dz, nf) - 1], 0.0)
    return w.min(), w.max()


def tip_deflection_percent(K, F, prob):
    """K_ff u = F_f; the probe's z deflection in percent of 5.02."""
    import scipy.sparse.linalg as spl
    nf = prob["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), F[:nf])
    d = prob["dofnums"][prob["probe"], 2]
    return u[d - 1] / 5.02 * 100


def surface_load(xyz, conn, dof, qz):
    """Consistent nodal loads of a uniform z traction (FinEtools distribloads
    with TriRule(3) on triangles / GaussRule(2,2) on quads)."""
    F = np.zeros(int(dof.max()))
    g = 0.577350269189626
    for e in range(conn.shape[0]):
        X = xyz[conn[e] - 1]
        if conn.shape[1] == 3:
            A = 0.5 * np.linalg.norm(np.cross(X[1] - X[0], X[2] - X[0]))
            for a in range(3):
                F[dof[conn[e, a] - 1, 2] - 1] += qz * A / 3
        else:
            for xi, eta in [(-g, -g), (-g, g), (g, -g), (g, g)]:
                N = 0.25 * np.array([(1 - xi) * (1 - eta), (1 + xi) * (1 - eta),
                                     (1 + xi) * (1 + eta), (1 - xi) * (1 + eta)])
                dN = 0.25 * np.array([[-(1 - eta), -(1 - xi)], [(1 - eta), -(1 + xi)],
                                      [(1 + eta), (1 + xi)], [-(1 + eta), (1 - xi)]])
                J = X.T @ dN
                Jac = np.linalg.norm(np.cross(J[:, 0], J[:, 1]))
                for a in range(4):
                    F[dof[conn[e, a] - 1, 2] - 1] += qz * N[a] * Jac
    return F


def solve_probe(K, prob):
    """K_ff u = F_f (solve_blocked! with zero prescribed values); returns the
    probe's transverse deflection as percent of -0.3024."""
    import scipy.sparse.linalg as spl
    nf = prob["nfree"]
    Kff = K[:nf, :nf].tocsc()
    u = spl.spsolve(Kff, prob["F"][:nf])
    d = prob["dofnums"][prob["probe"], 2]
    return (u[d - 1] if d <= nf else 0.0) / -0.3024 * 100


def jittered_plate(n, quads, side=1.0, jitter=0.2, seed=0, wavy=0.0, clamp_x0=True):
    """Seeded synthetic plate: n x n quads (or 2 n^2 triangles) on
    [0,side]^2, interior nodes jittered U(+-jitter*h), z = wavy*sin(pi x)
    sin(pi y); edge x = 0 clamped."""
    zf = None
    if wavy:
        zf = lambda x, y: wavy * np.sin(np.pi * x / side) * np.sin(np.pi * y / side)
    xyz, connq = mesh.jittered_plate_q(n, side, jitter, seed, zf)
    conn = connq if quads else mesh.quads_to_triangles(connq)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    if clamp_x0:
        fixed[np.abs(xyz[:, 0]) < 1e-12 * side, :] = True
    dof, nfree = mesh.numberdofs(fixed)
    return xyz, conn, dof, nfree


def cross_ply_groups(angles=(0, 90, 90, 0), ply_t=0.25e-3, E1=140e9, E2=10e9, G12=5e9, G13=5e9,
                     G23=3.5e9, nu12=0.3, rho=1600.0, csmat=None):
    """Plies of one layup (CompositeLayupModule.Ply, src/CompositeLayupModule.jl:71-97):
    list of dicts with the ply plane-stress Dps, transverse Dts, thickness,
    angle and density."""
    from flexshell import materials
    mat = materials.lamina_material(rho, E1, E2, nu12, G12, G13, G23)
    Dps, Dts = materials.shell_material_stiffness(mat)
    return [dict(Dps=Dps, Dts=Dts, thickness=ply_t, angle=a, rho=rho) for a in angles]


def barbero_plate(quads, n=8):
    """Barbero Example 3.1 [0/90] plate under opposite in-plane edge loads,
    test/test_composite_shell_statics.jl:14-97 (T3FFComp) and
    test/test_composite_shell_statics_q4rs.jl (Q4RSComp).  Returns the mesh,
    dofs, loads and the ply list."""
    from flexshell import materials
    ax = ay = 2.0
    E1, E2, G12, nu12, G23 = 133860e6, 7706e6, 4306e6, 0.301, 2760e6
    t = 0.010
    tol = ax / n / 100
    mat = materials.lamina_material(E1, E2, nu12, G12, G12, G23)
    Dps, Dts = materials.shell_material_stiffness(mat)
    plies = [dict(Dps=Dps, Dts=Dts, thickness=t / 2, angle=0.0, rho=0.0),
             dict(Dps=Dps, Dts=Dts, thickness=t / 2, angle=90.0, rho=0.0)]
    xy, conn = mesh.Q4block(ax, ay, n, n) if quads else mesh.T3block(ax, ay, n, n)
    xyz = mesh.xyz3(xy)
    inf = np.inf
    fixed = np.zeros((xyz.shape[0], 6), bool)
    l1 = mesh.selectnode(xyz, [ax, ax, 0, 0, -inf, inf], tol) - 1
    fixed[l1, 0:3] = True
    l1 = mesh.selectnode(xyz, [0, 0, 0, 0, -inf, inf], tol) - 1
    fixed[l1, 1] = True
    x, y = xyz[:, 0], xyz[:, 1]
    bnd = (np.abs(x) < tol) | (np.abs(x - ax) < tol) | (np.abs(y) < tol) | (np.abs(y - ay) < tol)
    fixed[bnd, 2] = True
    dof, nfree = mesh.numberdofs(fixed)
    # edge loads: q = +-0.1 MPa * t per unit length in y on the edges y = 0 and y = ay
    F = np.zeros(int(dof.max()))
    q = 0.1e6 * t
    xs = np.linspace(0.0, ax, n + 1)
    for yy, sgn in ((0.0, 1.0), (ay, -1.0)):
        nodes = [int(np.argmin(np.abs(x - xv) + np.abs(y - yy))) for xv in xs]
        for k in range(n):
            Le = xs[k + 1] - xs[k]
            for nd in (nodes[k], nodes[k + 1]):
                F[dof[nd, 1] - 1] += sgn * q * Le / 2
    # the same loads as the reference builds them: the L2 edges of meshboundary
    # on y = 0 and y = ay, GaussRule(1, 2), distribloads with m = 1
    bfes = mesh.meshboundary(conn)
    edge_loads = [(bfes[mesh.selectelem(xyz, bfes, [-inf, inf, yy, yy, 0, 0], tol)],
                   np.array([0, sgn * q, 0, 0, 0, 0.0])) for yy, sgn in ((0.0, 1.0), (ay, -1.0))]
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, plies=plies, F=F, thickness=t,
                edge_loads=edge_loads)


# test/test_composite_shell_statics.jl:97, test/test_composite_shell_statics_q4rs.jl:97
BARBERO_T3_UZMAX_MM = 0.22004349767718365
BARBERO_Q4_UZMAX_MM = 0.2278585006007462


def barbero_example(quads, example):
    """The layered plates of test/test_composite_shell_statics.jl and
    test/test_composite_shell_statics_q4rs.jl solved under edge loads built as
    the reference builds them (meshboundary, selectelem, GaussRule(1, 2),
    distribloads with m = 1):

    * "3.1x10": Barbero Example 3.1 with ten [0/90] pairs (:117-200), max w;
    * "3.3": Barbero Example 3.3, [+45/-45/0/0/-45/+45] plies of 1 mm pulled by
      +-200 N/mm in x on the edges x = 0 and x = ax (:234-323), max u;
    * "r+", "r-": [90/0] plies pulled (+) or pushed (-) in x on the edges
      x = 0 and x = ax (:870-954), max or min w;
    * "rot+", "rot-": the same plate turned into the y-z plane, (x, y, z) ->
      (z, x, y), with the layup csys columns (0,1,0), (0,0,1), (1,0,0) and the
      loads in z on the edges z = 0 and z = ax (:978-1075), max or min u;
    * "p0/90", "p-45/45": a 1 m square, 50 x 50, [0/90] or [-45/+45] plies,
      translations fixed on the boundary, a 1 MPa pressure over the surface
      (TriRule(1) / GaussRule(2, 2), m = 2; :683-753, :774-844), min w.

    Returns the mesh, dofs, plies, the edge loads (L2 connectivity, force
    intensity) or the surface load (its rule's code and intensity), the
    displacement component of the answer and the answer in mm."""
    from flexshell import materials
    if example.startswith("p"):
        return _barbero_pressure(quads, example)
    ax = ay = 2.0
    n = 8
    tol = ax / n / 100
    inf = np.inf
    csmat = np.eye(3)
    if example == "3.1x10":
        E1, E2, G12, nu12, G23 = 133860e6, 7706e6, 4306e6, 0.301, 2760e6
        t = 0.010
        angles = [0.0, 90.0] * 10
        ply_t = t / 20
    elif example.startswith("r"):
        E1, E2, G12, nu12, G23 = 133860e6, 7706e6, 4306e6, 0.301, 2760e6
        t = 0.010
        angles = [90.0, 0.0]
        ply_t = t / 2
        if example.startswith("rot"):
            csmat = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0.0]])
    else:
        E1, E2, G12, nu12, G23 = 37880e6, 9407e6, 3405e6, 0.299, 3308e6
        angles = [45.0, -45.0, 0.0, 0.0, -45.0, 45.0]
        ply_t = 1e-3
        t = ply_t * 6
    mat = materials.lamina_material(E1, E2, nu12, G12, G12, G23)
    Dps, Dts = materials.shell_material_stiffness(mat)
    plies = [dict(Dps=Dps, Dts=Dts, thickness=ply_t, angle=a, rho=0.0) for a in angles]
    xy, conn = mesh.Q4block(ax, ay, n, n) if quads else mesh.T3block(ax, ay, n, n)
    xyz = mesh.xyz3(xy)
    rot = example.startswith("rot")
    if rot:
        xyz = xyz[:, [2, 0, 1]].copy()
    fixed = np.zeros((xyz.shape[0], 6), bool)
    if rot:
        pin, roller = [0, 0, 0, 0, 0, 0], [0, 0, 0, 0, ax, ax]
    elif example == "3.1x10" or example.startswith("r"):
        pin, roller = [ax, ax, 0, 0, -inf, inf], [0, 0, 0, 0, -inf, inf]
    else:
        pin, roller = [0, 0, 0, 0, -inf, inf], [ax, ax, 0, 0, -inf, inf]
    fixed[mesh.selectnode(xyz, pin, tol) - 1, 0:3] = True
    fixed[mesh.selectnode(xyz, roller, tol) - 1, 1] = True
    bfes = mesh.meshboundary(conn)
    fixed[np.unique(bfes) - 1, 0 if rot else 2] = True  # connectednodes(meshboundary(fes))
    dof, nfree = mesh.numberdofs(fixed)
    extreme = "max"
    if example.startswith("r"):
        lm = 1.0 if example.endswith("+") else -1.0
        q = 0.1e6 * t * lm
        extreme = "max" if lm > 0 else "min"
        # the Q4RS file's values as printed there (:951-953, :1067-1069)
        ref = lm * ((0.22785850060074 if not rot else (0.22785850060 if lm < 0 else 0.227858500600))
                    if quads else 0.22004349767718365)
        if rot:
            boxes = [([0, 0, -inf, inf, ax, ax], [0, 0, q]), ([0, 0, -inf, inf, 0, 0], [0, 0, -q])]
            comp = 0
        else:
            boxes = [([0, 0, -inf, inf, 0, 0], [q, 0, 0]), ([ax, ax, -inf, inf, 0, 0], [-q, 0, 0])]
            comp = 2
        edge_loads = [(bfes[mesh.selectelem(xyz, bfes, b, tol)], np.array(f + [0, 0, 0.0])) for b, f in boxes]
        return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, plies=plies, thickness=t, csmat=csmat,
                    edge_loads=edge_loads, surface_load=None, comp=comp, ref=ref, extreme=extreme)
    if example == "3.1x10":
        q = 0.1e6 * t
        boxes = [([-inf, inf, 0, 0, 0, 0], [0, q]), ([-inf, inf, ay, ay, 0, 0], [0, -q])]
        comp, ref = 2, (0.010650045488315574 if quads else 0.010276258430770539)
    else:
        q = 200e3
        boxes = [([0, 0, -inf, inf, 0, 0], [-q, 0]), ([ax, ax, -inf, inf, 0, 0], [q, 0])]
        comp, ref = 0, 3.3161098653904544
    edge_loads = [(bfes[mesh.selectelem(xyz, bfes, b, tol)], np.array(f + [0, 0, 0, 0.0])) for b, f in boxes]
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, plies=plies, thickness=t, csmat=csmat,
                edge_loads=edge_loads, surface_load=None, comp=comp, ref=ref, extreme=extreme)


def _barbero_pressure(quads, example):
    from flexshell import materials
    ax = ay = 1.0
    n = 50
    tol = ax / n / 100
    E1, E2, G12, nu12, G23 = 133860e6, 7706e6, 4306e6, 0.301, 2760e6
    t = 0.010
    angles = [0.0, 90.0] if example == "p0/90" else [-45.0, 45.0]
    mat = materials.lamina_material(E1, E2, nu12, G12, G12, G23)
    Dps, Dts = materials.shell_material_stiffness(mat)
    plies = [dict(Dps=Dps, Dts=Dts, thickness=t / 2, angle=a, rho=0.0) for a in angles]
    xy, conn = mesh.Q4block(ax, ay, n, n) if quads else mesh.T3block(ax, ay, n, n)
    xyz = mesh.xyz3(xy)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[np.unique(mesh.meshboundary(conn)) - 1, 0:3] = True
    dof, nfree = mesh.numberdofs(fixed)
    refs = {("p0/90", False): -1502.0324040447633, ("p0/90", True): -1503.4206439821,
            ("p-45/45", False): -1176.8346659735575, ("p-45/45", True): -1177.349547131}
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, plies=plies, thickness=t, csmat=np.eye(3),
                edge_loads=[],
                surface_load=(2 if quads else 1, np.array([0, 0, -1.0e6, 0, 0, 0])), comp=2,
                ref=refs[(example, quads)], extreme="min")


def sacco_and_sandwich(quads, example):
    """Pressure-loaded layered plates of test/test_composite_shell_statics.jl
    (T3FFComp) and its Q4RS file (Q4RSComp), TriRule(1) / GaussRule(2, 2)
    surface loads with m = 2:

    * "sacco": [0/90] square, a = 250 mm, t = a/10, E1 = 100 GPa, E2 = E1/25,
      simple supports by edges (:1099-1183); two answers, max w and max u
      times 100 E2 / (q t (a/t)^4);
    * "sandwich": Barbero Example 3.7, faces 0.7112 mm over a 19.05 mm core of
      another material, translations fixed on the boundary (:1210-1282); max w.

    Returns the problem with its list of answers (component, extreme, scale,
    reference value)."""
    from flexshell import materials
    inf = np.inf
    if example == "sacco":
        a, n = 0.25, 8
        E1 = 100e9
        E2 = E1 / 25
        mat = materials.lamina_material(E1, E2, 0.25, E2 * 0.5, E2 * 0.5, E2 * 0.2)
        Dps, Dts = materials.shell_material_stiffness(mat)
        t = a / 10
        plies = [dict(Dps=Dps, Dts=Dts, thickness=t / 2, angle=ang, rho=0.0) for ang in (0.0, 90.0)]
        q = 10.0e3
    else:
        a, n = 2 * 0.127, 18
        face = materials.lamina_material(68947.57e6, 27579.03e6, 0.3, 12927.67e6, 12927.67e6, 12927.67e6)
        core = materials.lamina_material(0.068948e6, 0.068948e6, 0.0, 0.068948e6, 209.6e6, 82.737e6)
        tf, tc = 0.7112e-3, 19.05e-3
        plies = []
        for m_, tp in ((face, tf), (core, tc), (face, tf)):
            Dps, Dts = materials.shell_material_stiffness(m_)
            plies.append(dict(Dps=Dps, Dts=Dts, thickness=tp, angle=0.0, rho=0.0))
        t = 2 * tf + tc
        q = 0.689476e6
    tol = a / n / 100
    xy, conn = mesh.Q4block(a, a, n, n) if quads else mesh.T3block(a, a, n, n)
    xyz = mesh.xyz3(xy)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    bnd = np.unique(mesh.meshboundary(conn)) - 1
    if example == "sacco":
        for box, comps in (([0, 0, -inf, inf, 0, 0], [1, 3]), ([a, a, -inf, inf, 0, 0], [1, 3]),
                           ([-inf, inf, 0, 0, 0, 0], [0, 4]), ([-inf, inf, a, a, 0, 0], [0, 4])):
            fixed[np.ix_(mesh.selectnode(xyz, box, tol) - 1, comps)] = True
        fixed[bnd, 2] = True
        sc = 100 * E2 / (q * t * (a / t) ** 4)
        answers = [(2, "max", sc, 2.0134037916683 if quads else 1.9529295928169146),
                   (0, "max", sc, 0.128716225 if quads else 0.12375916912652352)]
    else:
        fixed[bnd, 0:3] = True
        answers = [(2, "max", 1e3, 3.201455454 if quads else 3.2024601774900674)]
    dof, nfree = mesh.numberdofs(fixed)
    return dict(xyz=xyz, conn=conn, dofnums=dof, nfree=nfree, plies=plies, thickness=t, csmat=np.eye(3),
                edge_loads=[], surface_load=(2 if quads else 1, np.array([0, 0, q, 0, 0, 0])), answers=answers)


def extreme_displacements(K, F, d):
    """K_ff u = F_f; (value, reference) of every answer of d["answers"]."""
    import scipy.sparse.linalg as spl
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), F[:nf])
    out = []
    for comp, ext, scale, ref in d["answers"]:
        dc = d["dofnums"][:, comp]
        v = np.where(dc <= nf, u[np.minimum(dc, nf) - 1], 0.0)
        out.append(((v.max() if ext == "max" else v.min()) * scale, ref))
    return out


def max_displacement_mm(K, F, d):
    """K_ff u = F_f; the largest (d["extreme"] "max") or smallest ("min")
    nodal displacement of component d["comp"], in mm."""
    import scipy.sparse.linalg as spl
    nf = d["nfree"]
    u = spl.spsolve(K[:nf, :nf].tocsc(), F[:nf])
    dc = d["dofnums"][:, d["comp"]]
    v = np.where(dc <= nf, u[np.minimum(dc, nf) - 1], 0.0)
    return (v.max() if d["extreme"] == "max" else v.min()) / 1e-3


def c4_plate(n, side=1.0):
    """The layered-plate configuration: n x n Q4 on a flat square (side 1 m),
    [0/90/90/0] plies of 0.25 mm (E1 140 GPa, E2 10 GPa, G12 = G13 5 GPa, G23
    3.5 GPa, nu12 0.3, rho 1600), cartesian layup csys, simply supported
    (w = 0 on the boundary) with the in-plane rigid-body motion restrained
    (u = v = 0 at (0, 0), v = 0 at (side, 0)): left free, those three zero
    modes would be lifted by any rounding of the membrane stiffness into the
    range of the lowest bending modes."""
    xy, conn = mesh.Q4block(side, side, n, n)
    xyz = mesh.xyz3(xy)
    x, y = xyz[:, 0], xyz[:, 1]
    tol = side / n / 100
    bnd = (np.abs(x) < tol) | (np.abs(x - side) < tol) | (np.abs(y) < tol) | (np.abs(y - side) < tol)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    fixed[bnd, 2] = True
    c0 = int(np.argmin(np.abs(x) + np.abs(y)))
    c1 = int(np.argmin(np.abs(x - side) + np.abs(y)))
    fixed[c0, 0] = fixed[c0, 1] = fixed[c1, 1] = True
    dof, nfree = mesh.numberdofs(fixed)
    return xyz, conn, dof, nfree, cross_ply_groups((0, 90, 90, 0))


def lowest_eigenvalues(K, M, nev=20, sigma=-1.0):
    """The nev lowest eigenvalues of (K, M) by shift-invert Lanczos (ARPACK,
    as the reference's eigs) about `sigma`."""
    import scipy.sparse.linalg as spl
    w = spl.eigsh(K.tocsc(), k=nev, M=M.tocsc(), sigma=sigma, which="LM", return_eigenvectors=False,
                  tol=1e-12)
    return np.sort(w)

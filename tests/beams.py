"""Beam problems of the reference test suite, driven through an "engine".

An engine offers the FEMMCorotBeam calls (stiffness, geostiffness, mass,
gyroscopic, restoringforce, distribloads_global) on numpy inputs and returns
the free-free blocks; `OracleBeams` runs them with the CPU oracle and
`GpuBeams` with the library.  The drivers restate the reference tests:

- L-frame modal analysis, test/test_beam_modal.jl:17-77 (module mmodal1)
- cantilever buckling, test/test_beam_buckling.jl:18-87 (module mbuckling1)
- fast spinning top, test/test_beam_dyn.jl:20-253 (module mfasttoptest1)
"""
import numpy as np
import scipy.linalg as sla

from flexshell import beam as B
from flexshell.femm import NodalField, SysmatAssemblerFFBlock, SysmatAssemblerSparseSymm

# reference answers
LFRAME_FREQS = [11.2732, 30.5269]               # test/test_beam_modal.jl:30, rtol 3e-5 (:74)
BUCKLING_FACTORS = [48.5475, 124.1839]          # test/test_beam_buckling.jl:30, rtol 1e-3 (:85)
FAST_TOP_TIPX = [
    0.0, 7.436031085824281e-7, 0.11777019275816547, 0.8203709506659435, 2.241864039281919,
    3.9679895248072063, 5.3454217754301885, 5.971372979336259, 5.994274006124595,
    5.998838219173172, 6.562336269473291, 7.816659235667364, 9.346281101346545,
    10.499101141896105, 10.875849911112233, 10.628929261212697, 10.345322488144156,
    10.602025422687818, 11.529299245601559, 12.710964257026657, 13.496913529329909,
    13.492271339298975, 12.854269845420365, 12.172880227196368, 12.025322964890227,
    12.540504127222404, 13.301744975038586]     # test/test_beam_dyn.jl:195-223
FAST_TOP_TIPY = [
    -11.995000624962799, -11.99507329138783, -12.34434321937684, -13.092699071921164,
    -13.606709453527161, -13.384277801594491, -12.433899377302394, -11.269034682594993,
    -10.521805428897146, -10.467440913151172, -10.818091285108137, -10.941387824929802,
    -10.338997425035933, -9.024387391352876, -7.51482956095552, -6.443555337060203,
    -6.084606620045228, -6.148711597765479, -6.004002866512018, -5.155146068191021,
    -3.6197117072489498, -1.9179359415572481, -0.6834506841073384, -0.18854220120395482,
    -0.1419789099985156, 0.08825549466116911, 0.9953416189668296]   # :224-251


class Material:
    def __init__(self, E, nu, rho=0.0):
        self.E, self.nu, self.rho = E, nu, rho

    def massdensity(self):
        return self.rho


class OracleBeams:
    """The CPU oracle behind the engine interface (free-free blocks)."""

    def __init__(self, xyz, conn, sections, mat):
        from oracle import oracle as O
        self.o = O
        self.b = O.Beam(xyz, conn, sections, mat.E, mat.nu, mat.rho)
        self.conn = conn

    def _mat(self, which, dofnums, nfree, **kw):
        return self.b.matrix(which, dofnums, nfree, mode=self.o.DROP_ZEROS, **kw)

    def stiffness(self, u1, R1, dofnums, nfree):
        return self._mat(self.o.BEAM_STIFFNESS, dofnums, nfree, u1=u1, R1=R1)

    def geostiffness(self, u1, R1, dofnums, nfree):
        return self._mat(self.o.BEAM_GEOSTIFFNESS, dofnums, nfree, u1=u1, R1=R1)

    def mass(self, u1, R1, dofnums, nfree, mass_type=1):
        return self._mat(self.o.BEAM_MASS, dofnums, nfree, u1=u1, R1=R1, mass_type=mass_type)

    def gyroscopic(self, u1, R1, v1, dofnums, nfree, mass_type=1):
        return self._mat(self.o.BEAM_GYROSCOPIC, dofnums, nfree, u1=u1, R1=R1, v1=v1,
                         mass_type=mass_type)

    def restoringforce(self, u1, R1, dofnums, nfree):
        return self.b.vector(self.o.BEAM_RESTORING, dofnums, nfree, u1=u1, R1=R1)

    def distribloads(self, u1, R1, dofnums, nfree, q):
        return self.b.vector(self.o.BEAM_DISTRIBLOAD, dofnums, nfree, u1=u1, R1=R1, q=q)


class GpuBeams:
    """FEMMCorotBeam (libflexshell) behind the engine interface."""

    def __init__(self, xyz, conn, sections, mat, device=0):
        self.femm = B.FEMMCorotBeam(conn, sections, mat, device)
        self.geom0 = NodalField(xyz)
        self.dchi = NodalField(np.zeros((xyz.shape[0], 6)))

    def _prep(self, dofnums, nfree):
        self.dchi.dofnums = np.asfortranarray(dofnums)
        self.dchi.nfreedofs = nfree
        return SysmatAssemblerFFBlock(SysmatAssemblerSparseSymm(), nfree)

    def stiffness(self, u1, R1, dofnums, nfree):
        a = self._prep(dofnums, nfree)
        return self.femm.stiffness(a, self.geom0, u1, R1, self.dchi)

    def geostiffness(self, u1, R1, dofnums, nfree):
        a = self._prep(dofnums, nfree)
        return self.femm.geostiffness(a, self.geom0, u1, R1, self.dchi)

    def mass(self, u1, R1, dofnums, nfree, mass_type=1):
        a = self._prep(dofnums, nfree)
        return self.femm.mass(a, self.geom0, u1, R1, self.dchi, mass_type=mass_type)

    def gyroscopic(self, u1, R1, v1, dofnums, nfree, mass_type=1):
        a = self._prep(dofnums, nfree)
        return self.femm.gyroscopic(a, self.geom0, u1, R1, v1, self.dchi, mass_type=mass_type)

    def restoringforce(self, u1, R1, dofnums, nfree):
        self._prep(dofnums, nfree)
        return self.femm.restoringforce(self.geom0, u1, R1, self.dchi)[:nfree]

    def distribloads(self, u1, R1, dofnums, nfree, q):
        self._prep(dofnums, nfree)
        return self.femm.distribloads_global(self.geom0, u1, R1, self.dchi, q)[:nfree]

    def close(self):
        self.femm.close()


def numberdofs(nnodes, fixed):
    """numberdofs!: free dofs first (node-major), then the fixed ones."""
    from flexshell import mesh
    d, nf = mesh.numberdofs(fixed)
    return np.asfortranarray(d), nf


def lattice_frame(n=3, seed=0):
    """Beams along the edges of a jittered n x n x n lattice, random sections
    (Bernoulli and Timoshenko), random deformed state (u, R, v)."""
    rng = np.random.default_rng(seed)
    g = np.arange(n, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.column_stack([X.ravel(), Y.ravel(), Z.ravel()]) * 2.0
    xyz += rng.uniform(-0.2, 0.2, xyz.shape)
    idx = np.arange(n ** 3).reshape(n, n, n) + 1
    conn = []
    for ax in range(3):
        a = np.moveaxis(idx, ax, 0)
        conn += list(zip(a[:-1].ravel(), a[1:].ravel()))
    conn = np.array(conn, dtype=np.int64)
    ne, nn = conn.shape[0], xyz.shape[0]
    sec = np.zeros((ne, 10))
    sec[:, 0] = rng.uniform(0.5, 2.0, ne)
    sec[:, 2] = rng.uniform(0.05, 0.3, ne)
    sec[:, 3] = rng.uniform(0.05, 0.3, ne)
    sec[:, 1] = sec[:, 2] + sec[:, 3]
    sec[:, 4] = rng.uniform(0.05, 0.4, ne)
    tim = rng.random(ne) < 0.5
    sec[:, 5] = np.where(tim, sec[:, 0] * 5 / 6, np.inf)
    sec[:, 6] = np.where(tim, sec[:, 0] * 5 / 6, np.inf)
    sec[:, 7:] = rng.normal(size=(ne, 3))
    u1 = rng.uniform(-0.05, 0.05, (nn, 3))
    R1 = np.stack([B.rotmat3(rng.normal(scale=0.3, size=3)).flatten(order="F") for _ in range(nn)])
    v1 = rng.normal(size=(nn, 6))
    fixed = np.zeros((nn, 6), dtype=bool)
    fixed[0, :] = True
    fixed[1, :3] = True
    dof, nf = numberdofs(nn, fixed)
    return xyz, conn, sec, u1, R1, v1, dof, nf


# ---------------------------------------------------------------------------
def lframe(n=4):
    """Mesh of the L frame of test/test_beam_modal.jl:22-41."""
    b, h, L = 3.0, 30.0, 240.0
    cs = B.CrossSectionRectangle(b, h, [0.0, 1.0, 0.0])
    m1 = B.frame_member([[0, 0, L], [L, 0, L]], n, cs)
    m2 = B.frame_member([[L, 0, L], [L, 0, 0]], n, cs)
    xyz, conn, sec = B.merge_members([m1, m2], tolerance=L / 10000)
    return xyz, conn, sec, Material(71240.0, 0.31, 5e-9), L


def lframe_modal(make_engine, mass_type=1, n=4):
    """Two lowest frequencies [Hz] of the clamped L frame.  The test calls mass()
    without a mass_type (test/test_beam_modal.jl:64), i.e. the default consistent
    mass with rotary inertia."""
    xyz, conn, sec, mat, L = lframe(n)
    fixed = np.zeros((xyz.shape[0], 6), dtype=bool)
    fixed[B.selectnode(xyz, [0, 0, 0, 0, L, L], L / 10000) - 1, :] = True
    dof, nf = numberdofs(xyz.shape[0], fixed)
    eng = make_engine(xyz, conn, sec, mat)
    nn = xyz.shape[0]
    u0, R0 = np.zeros((nn, 3)), B.initial_Rfield(nn).values
    K = eng.stiffness(u0, R0, dof, nf).toarray()
    M = eng.mass(u0, R0, dof, nf, mass_type).toarray()
    # eigs(K, M; which = :SM) with a singular lumped M: largest mu of M x = mu K x
    mu = sla.eigh(M, K, eigvals_only=True)
    lam = 1.0 / np.sort(mu[mu > 0])[::-1]
    return np.sqrt(lam[:2]) / (2 * np.pi), eng


def cantilever_buckling(make_engine, n=32):
    """Buckling factors of the tip-loaded cantilever (test/test_beam_buckling.jl:18-87)."""
    E, nu, L, b, h = 1e6, 0.3, 30.0, 0.5, 4.0
    magn = -0.2056167583560 * 1e4 / L ** 2
    magn_scale = 1000
    cs = B.CrossSectionRectangle(b, h, [-1.0, 0.0, 0.0])
    xyz, conn, sec = B.merge_members([B.frame_member([[0, 0, 0], [0, 0, L]], n, cs)],
                                     tolerance=L / 10000)
    nn = xyz.shape[0]
    fixed = np.zeros((nn, 6), dtype=bool)
    fixed[B.selectnode(xyz, [0, 0, 0, 0, 0, 0], L / 10000) - 1, :] = True
    dof, nf = numberdofs(nn, fixed)
    eng = make_engine(xyz, conn, sec, Material(E, nu))
    u0, R0 = np.zeros((nn, 3)), B.initial_Rfield(nn)
    K = eng.stiffness(u0, R0.values, dof, nf).toarray()
    # point load at the tip (distribloads on a point set): dof 2 of the tip node
    tip = B.selectnode(xyz, [0, 0, 0, 0, L, L], L / 10000)[0]
    F = np.zeros(nf)
    F[dof[tip - 1, 1] - 1] = -magn * b * h / magn_scale
    uf = np.linalg.solve(K, F)
    dchi = NodalField(np.zeros((nn, 6)))
    for i in range(nn):
        for k in range(6):
            if dof[i, k] <= nf:
                dchi.values[i, k] = uf[dof[i, k] - 1]
    u0 = dchi.values[:, :3].copy()
    B.update_rotation_field(R0, dchi)
    Kg = eng.geostiffness(u0, R0.values, dof, nf).toarray()
    # eigs(-Kg_ff, K_ff; which = :LM): largest |d| of -Kg x = d K x
    d = sla.eigh(-Kg, K, eigvals_only=True)
    d = d[np.argsort(-np.abs(d))]
    fs = 1.0 / d / magn_scale
    return np.abs(fs[1:3]), eng


def fast_top(make_engine, tend=0.8, record_every=50):
    """Newmark / Newton loop of the fast top (test/test_beam_dyn.jl:20-253).
    Returns the recorded tip x and y coordinates."""
    E, nu, rho = 71240.0, 0.31, 2.7e-9
    W = H = 60.0
    Length = 4 * W
    Omega0 = 313 * np.pi
    R0 = B.rotmat3([0.05, 0, 0])
    g = 9.81e3
    q = np.array([0.0, 0.0, -g * W * H * rho])
    maxit = 12
    dt = min(2 * np.pi / abs(Omega0) / 10, 0.005)
    ng = 1 / 2
    nb = 1 / 4 * (1 / 2 + ng) ** 2
    cs = B.CrossSectionRectangle(W, W, [1.0, 0.0, 0.0])
    spin = R0 @ np.array([0.0, 0.0, Omega0])
    X = np.array([[0.0, 0.0, 0.0], R0 @ np.array([0.0, 0.0, Length])])
    n = 8
    tol = Length / n / 100
    xyz, conn, sec = B.merge_members([B.frame_member(X, n, cs)], tolerance=tol)
    nn = xyz.shape[0]
    support = B.selectnode(xyz, [X[0, 0], X[0, 0], X[0, 1], X[0, 1], X[0, 2], X[0, 2]], tol)
    tipn = B.selectnode(xyz, [X[1, 0], X[1, 0], X[1, 1], X[1, 1], X[1, 2], X[1, 2]], tol)
    fixed = np.zeros((nn, 6), dtype=bool)
    fixed[support - 1, :3] = True
    dof, nf = numberdofs(nn, fixed)
    eng = make_engine(xyz, conn, sec, Material(E, nu, rho))

    free = dof <= nf
    order = dof[free] - 1                      # free entries of a (nn, 6) array -> system index

    def gather(a):
        v = np.zeros(nf)
        v[order] = a[free]
        return v

    def scatter(v):
        a = np.zeros((nn, 6))
        a[free] = v[order]
        return a

    utol = 1e-13 * nf
    u0 = np.zeros((nn, 3))
    Rf0 = B.initial_Rfield(nn)
    v0 = np.zeros((nn, 6))
    v0[:, 3:6] = spin
    a0 = np.zeros((nn, 6))
    u1 = u0.copy()
    Rf1 = NodalField(Rf0.values.copy())
    tipx, tipy = [X[1, 0]], [X[1, 1]]
    t, step = 0.0, 0
    while t <= tend:
        t += dt
        u1[:] = u0
        Rf1.values[:] = Rf0.values
        stepdchi = np.zeros((nn, 6))
        a1 = -(1 / nb / dt) * v0 - (1 / 2 - nb) / nb * a0
        v1 = v0 + dt * ((1 - ng) * a0 + ng * a1)
        v0v, a0v = gather(v0), gather(a0)
        dchipv = dt * v0v + (dt ** 2 / 2 * (1 - 2 * nb)) * a0v
        vpv = v0v + (dt * (1 - ng)) * a0v
        it = 1
        while True:
            F = eng.distribloads(u1, Rf1.values, dof, nf, q)
            Fr = eng.restoringforce(u1, Rf1.values, dof, nf)
            rhs = F + Fr
            K = eng.stiffness(u1, Rf1.values, dof, nf)
            M = eng.mass(u1, Rf1.values, dof, nf)
            G = eng.gyroscopic(u1, Rf1.values, v1, dof, nf)
            sv = gather(stepdchi)
            rhs = rhs + M @ ((-1 / (nb * dt ** 2)) * sv + (1 / (nb * dt ** 2)) * dchipv)
            rhs = rhs + G @ ((-ng / nb / dt) * sv + (ng / nb / dt) * dchipv - vpv)
            A = (K + (ng / nb / dt) * G + (1 / (nb * dt ** 2)) * M).toarray()
            dchi = NodalField(scatter(np.linalg.solve(A, rhs)))
            u1 += dchi.values[:, :3]
            stepdchi += dchi.values
            v1 = v1 + (ng / nb / dt) * dchi.values
            a1 = a1 + (1 / nb / dt ** 2) * dchi.values
            B.update_rotation_field(Rf1, dchi)
            if np.max(np.abs(dchi.values)) < utol:
                break
            if it > maxit:
                raise RuntimeError("Possible failed convergence")
            it += 1
        u0[:] = u1
        Rf0.values[:] = Rf1.values
        v0, a0 = v1, a1
        if step % record_every == 0:
            tipx.append(X[1, 0] + u1[tipn[0] - 1, 0])
            tipy.append(X[1, 1] + u1[tipn[0] - 1, 1])
        step += 1
    return np.array(tipx), np.array(tipy), eng

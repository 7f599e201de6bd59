"""The compensated sums of the FS_MIXED_COMP mode, run on the host.

csrc/fs_comp_sum.cuh holds the arithmetic behind the compensated mode's
accuracy: the element kernels' Dot2 (T3) and three-level (Q4) Gram sums on
packed float pairs, their (hi, lo) float-pair results, and the gather's
float-triple column sums rounded once to double.  The library compiles it to
packed FP32x2 instructions; a host compiler gets the same operations lane by
lane (tests/hostcheck).  These tests check each sum against the exact
rational value on ill-conditioned inputs, with error bounds derived for the
sums as written (u = 2^-24, gamma_k = k u / (1 - k u), S = sum of |terms|):

* Dot2 to a float pair (Ogita, Rump and Oishi, "Accurate sum and dot
  product", SIAM J. Sci. Comput. 26 (2005), with the final rounding left out
  since the pair keeps s + c): |err| <= gamma_{n+1}^2 S.
* Three levels: the product errors are summed once in float, the TwoSum
  errors of the compensation exactly: |err| <= 2.1 u gamma_{n+1} S.
* The gather's triple: the tail's float rounding, then one rounding to
  double: |err| <= 2^-52 |X| + 8 n^2 (n + 1) u^3 S.

Both dot-product bounds need Fast2Sum(s, c) to be exact, which holds while
|s| >= |c|: for a condition number S / |X| up to 1 / (4 gamma_{n+1}).  Below
the normal range the split of a product a b into p and its error is exact
only to half the subnormal spacing eta = 2^-149 (the instructions keep
subnormals, as IEEE arithmetic does on the host): an absolute 2 n eta is
added to the dot-product bounds.
Then the element matrices of the compensated path are checked against the
exact Gram of the same float rows with the same bounds, entry by entry, and
the thin layered plate's lowest eigenvalues are computed from them: the
reason the compensated mode exists, reproduced on the host.
"""
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O
from flexshell import _abi
from hostcheck import hostmath as HC
from test_hostcheck import _composite, _homog, _relmax

U = 2.0 ** -24
ETA = 2.0 ** -149


def _gamma(k):
    return k * U / (1 - k * U)


def _gen_dot(rng, n, cond):
    """Float32 vectors x, y whose dot product has about the condition number
    `cond` (the construction of Ogita, Rump and Oishi's GenDot): half the
    terms with exponents spread over log2(cond) / 2, the other half chosen to
    cancel the running exact sum."""
    b = max(1, int(round(np.log2(cond) / 2)))
    n2 = n // 2
    e = np.concatenate(([b], rng.integers(0, b + 1, n2 - 2), [0])) if n2 >= 2 else np.array([b])
    x = np.zeros(n, np.float32)
    y = np.zeros(n, np.float32)
    x[:n2] = ((2 * rng.random(n2) - 1) * 2.0 ** e).astype(np.float32)
    y[:n2] = ((2 * rng.random(n2) - 1) * 2.0 ** e).astype(np.float32)
    part = sum((Fraction(float(a)) * Fraction(float(c)) for a, c in zip(x[:n2], y[:n2])), Fraction(0))
    for i, ei in zip(range(n2, n), np.linspace(b, 0, n - n2)):
        x[i] = np.float32((2 * rng.random() - 1) * 2.0 ** ei)
        if x[i] == 0:
            x[i] = np.float32(1.0)
        y[i] = np.float32(((2 * rng.random() - 1) * 2.0 ** ei - float(part)) / float(x[i]))
        part += Fraction(float(x[i])) * Fraction(float(y[i]))
    p = rng.permutation(n)
    return x[p], y[p]


def _exact_dot(x, y):
    X = sum((Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y)), Fraction(0))
    S = sum((abs(Fraction(float(a)) * Fraction(float(b))) for a, b in zip(x, y)), Fraction(0))
    return X, S


def _pair_err(hl, X):
    return abs(Fraction(float(hl[0])) + Fraction(float(hl[1])) - X)


def _dot_bound(levels, n, S):
    g = _gamma(n + 1)
    return Fraction(g * g if levels == 2 else 2.1 * U * g) * S + Fraction(2 * n * ETA)


@pytest.mark.parametrize("levels", [2, 3])
@pytest.mark.parametrize("n", [9, 33])
def test_compensated_dot_error_bound(levels, n):
    # the pair (hi, lo) of an ill-conditioned dot product within the bound of
    # its summation depth, on both lanes; condition numbers 1 .. 1/(4 gamma)
    rng = np.random.default_rng(100 * levels + n)
    cmax = 1 / (4 * _gamma(n + 1))
    worst = 0.0
    for t in range(60):
        cond = float(np.exp(rng.uniform(0, np.log(cmax))))
        x, y0 = _gen_dot(rng, n, cond)
        _, y1 = _gen_dot(rng, n, cond)
        for y, hl in zip((y0, y1), HC.comp_dot(levels, x, y0, y1)):
            X, S = _exact_dot(x, y)
            if X == 0 or S / abs(X) > cmax:
                continue
            err = _pair_err(hl, X)
            bound = _dot_bound(levels, n, S)
            assert err <= bound, (levels, n, t, float(err / S))
            worst = max(worst, float(err / bound))
    assert worst > 0  # the inputs did exercise the compensation


@pytest.mark.parametrize("levels", [2, 3])
def test_compensated_dot_exact_cancellation(levels):
    # terms that cancel exactly (a second copy of each product, negated): the
    # result is within the bound of zero, far below plain float's n u S
    rng = np.random.default_rng(7 + levels)
    for t in range(40):
        h = int(rng.integers(3, 17))
        a = (rng.standard_normal(h) * 2.0 ** rng.integers(-20, 20, h)).astype(np.float32)
        b = (rng.standard_normal(h) * 2.0 ** rng.integers(-20, 20, h)).astype(np.float32)
        p = rng.permutation(2 * h)
        x = np.concatenate([a, a])[p]
        y = np.concatenate([b, -b])[p]
        hl, _ = HC.comp_dot(levels, x, y, y)
        X, S = _exact_dot(x, y)
        assert X == 0
        assert _pair_err(hl, X) <= 2 * _dot_bound(levels, 2 * h, S)


def test_dot2_and_three_levels_against_plain_float():
    # the depth matters where the terms are many: at 33 terms per entry (a Q4
    # element) the three-level sums' bound is 16 times below Dot2's, and both
    # beat plain float sums by orders of magnitude on the same inputs
    rng = np.random.default_rng(3)
    n = 33
    assert _dot_bound(2, n, Fraction(1)) > 16 * _dot_bound(3, n, Fraction(1))
    e2 = e3 = ef = Fraction(0)
    for t in range(40):
        x, y = _gen_dot(rng, n, 1e4)
        X, S = _exact_dot(x, y)
        (hl2, _), (hl3, _) = HC.comp_dot(2, x, y, y), HC.comp_dot(3, x, y, y)
        s = np.float32(0)
        for a, b in zip(x, y):
            s = np.float32(s + np.float32(a * b))
        e2 = max(e2, _pair_err(hl2, X) / S)
        e3 = max(e3, _pair_err(hl3, X) / S)
        ef = max(ef, abs(Fraction(float(s)) - X) / S)
    assert max(e2, e3) * 1e5 < ef


def _gen_pairs(rng, n, cond):
    """n normalised float pairs (hi, lo = the rounding of x - hi) of reals
    whose sum has about the condition number `cond`."""
    b = max(1, int(round(np.log2(cond))))
    xs = []
    part = Fraction(0)
    for i in range(n):
        ei = b if i == 0 else int(rng.integers(0, b + 1))
        v = Fraction((2 * rng.random() - 1) * 2.0 ** ei) * (1 + Fraction(int(rng.integers(1, 2 ** 20)), 2 ** 45))
        if i >= n // 2:
            v -= part * Fraction(int(rng.integers(1, 1000)), 1000)
        xs.append(v)
        part += v
    hi = np.array([np.float32(float(v)) for v in xs], np.float32)
    lo = np.array([np.float32(float(v - Fraction(float(h)))) for v, h in zip(xs, hi)], np.float32)
    return hi, lo


@pytest.mark.parametrize("n", [2, 6, 12, 24])
def test_gather_triple_sum_error_bound(n):
    # the gather's column sums of float pairs: within 2^-52 of the exact sum
    # plus the tail's u^3 term, on ill-conditioned sums of both lanes
    rng = np.random.default_rng(n)
    worst = 0.0
    for t in range(60):
        cond = float(np.exp(rng.uniform(0, np.log(1e12))))
        h0, l0 = _gen_pairs(rng, n, cond)
        h1, l1 = _gen_pairs(rng, n, cond)
        out = HC.triple_sum(np.stack([h0, h1]), np.stack([l0, l1]))
        for v, hi, lo in zip(out, (h0, h1), (l0, l1)):
            terms = [Fraction(float(a)) + Fraction(float(b)) for a, b in zip(hi, lo)]
            X = sum(terms, Fraction(0))
            S = sum((abs(q) for q in terms), Fraction(0))
            err = abs(Fraction(float(v)) - X)
            bound = Fraction(2.0 ** -52) * abs(X) + Fraction(8 * n * n * (n + 1) * U ** 3) * S
            assert err <= bound, (n, t, float(err), float(bound))
            worst = max(worst, float(err / bound))
    assert worst > 0


def _comp_cases():
    """(element type, xyz, conn, oracle problem, thickness, parameters, layup
    groups, element groups, rows per element)."""
    out = []
    for quads in (False, True):
        et, d, P, prm = _homog(quads)
        out.append((et, d["xyz"], d["conn"], P, d["thickness"], prm, None, None, 36 if quads else 11))
        et, xyz, conn, P, prm, g = _composite(quads)
        out.append((et, xyz, conn, P, 0.0, prm, [g], np.zeros(len(conn)), 36 if quads else 11))
    et, d, P, prm = _homog(False, tsf=1)  # T3 average K: 15 rows
    out.append((et, d["xyz"], d["conn"], P, d["thickness"], prm, None, None, 15))
    return out


@pytest.mark.parametrize("case", range(5), ids=["t3ff", "t3ffcomp", "q4rs", "q4rscomp", "t3ff_avgk"])
def test_comp_element_matrices_within_the_sums_bounds(case):
    # every entry of the compensated element matrices against the exact Gram
    # of the same float rows: within the Dot2 bound (T3) or the three-level
    # bound (Q4) plus the final rounding to double (the layered T3 plate has
    # entries near 1e-34, where the underflow term is the one that counts);
    # and against the oracle's FP64 matrices within the float rows' own error
    et, xyz, conn, P, th, prm, groups, eg, nrows = _comp_cases()[case]
    args = (xyz, conn, P.normals, P.valid, th, prm)
    kw = dict(groups=groups, egroup=eg)
    Kc = HC.element_matrices(et, _abi.FS_MIXED_COMP, *args, **kw)
    Kx = HC.element_matrices(et, 3, *args, **kw)
    Ka = HC.element_matrices(et, 4, *args, **kw)
    quads = conn.shape[1] == 4
    g = _gamma(nrows + 1)
    coef = 2.1 * U * g if quads else g * g
    bound = coef * Ka + 2.0 ** -52 * np.abs(Kx) + 2 * nrows * ETA
    err = np.abs(Kc - Kx)
    assert np.all(err <= bound)
    assert err.max() > 0 or Ka.max() == 0
    assert max(_relmax(Kc[e], Kx[e]) for e in range(len(Kc))) <= 1e-12
    Ko = P.element_stiffness()
    assert _relmax(Kc, Ko) <= 1e-6


@pytest.mark.parametrize("triangles,n,mixed_floor", [(False, 32, 1e-4), (True, 16, 1e-5)],
                         ids=["q4rscomp_32", "t3ffcomp_16"])
def test_layered_plate_eigenvalues_need_the_compensated_sums(triangles, n, mixed_floor):
    # the layered plate ([0/90/90/0], t/L = 0.001), as Q4RSComp quads or split
    # into T3FFComp triangles: element matrices from the kernels' own
    # arithmetic on the host, assembled in double, and the 20 lowest
    # eigenvalues with the oracle's lumped mass, against FP64.  Plain float
    # Gram sums (FS_MIXED) miss the 1e-6 target (their rounding is not of the
    # Gram form and acts as a spurious foundation under the bending modes;
    # measured Q4 2.0e-5 at 16 x 16 and 2.5e-3 at 32 x 32, T3 4.6e-5 at
    # 16 x 16); the compensated sums meet it (measured 6e-8 to 9.4e-8)
    import scipy.sparse as sp
    import problems as PB
    from flexshell import mesh
    xyz, conn, dof, nfree, plies = PB.c4_plate(n)
    et, stab = (O.T3FFCOMP, 5 / 12 / 1.5) if triangles else (O.Q4RSCOMP, 0.1)
    if triangles:
        conn = mesh.quads_to_triangles(conn)
    A, B, D, H, md, mi = O.laminate(plies)
    t = sum(p["thickness"] for p in plies)
    P = O.Problem(et, xyz, conn, dof, stab_c=stab,
                  groups=[dict(A=A, B=B, D=D, H=H, csmat=np.eye(3), thickness=t, mass=md, moi=mi)])
    P.compute_normals()
    g = _abi.make_group(A, B, D, H, np.eye(3), t, md, mi)
    prm = _abi.make_params(np.eye(3), np.eye(2), 0.0, t, stab_c=stab, quads=not triangles)
    M = P.assemble_scipy("M", O.KEEP_ZEROS, n=nfree)
    nd = 6 * conn.shape[1]
    dd = np.stack([np.concatenate([dof[a - 1] for a in e]) - 1 for e in conn])
    r, c = np.repeat(dd, nd, axis=1).ravel(), np.tile(dd, (1, nd)).ravel()
    keep = (r < nfree) & (c < nfree)

    def lowest(precision):
        Ke = HC.element_matrices(et, precision, xyz, conn, P.normals, P.valid, 0.0, prm,
                                 groups=[g], egroup=np.zeros(len(conn)))
        K = sp.csc_matrix((Ke.ravel()[keep], (r[keep], c[keep])), shape=(nfree, nfree))
        return PB.lowest_eigenvalues(K, M)

    w64 = lowest(_abi.FS_FP64)
    err = {p: np.max(np.abs(lowest(p) - w64) / np.abs(w64)) for p in (_abi.FS_MIXED, _abi.FS_MIXED_COMP)}
    assert err[_abi.FS_MIXED_COMP] <= 1e-6, err
    assert err[_abi.FS_MIXED] >= mixed_floor, err

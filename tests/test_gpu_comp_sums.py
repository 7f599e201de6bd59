"""The packed FP32x2 compensated sums on the GPU, bitwise against the host.

tests/test_comp_sums.py proves the error bounds of csrc/fs_comp_sum.cuh's
sums with the host's lane-by-lane IEEE binary32 arithmetic.  Those results
carry over to the kernels only if the packed instructions (add, sub, mul,
fma .rn .f32x2, no flush to zero) round each lane as IEEE does: here the
same header, built for sm_103a (tests/hostcheck/devcheck.cu), runs the
element kernels' Dot2 and three-level dot products and the gather's
float-triple column sums on inputs that reach ill-conditioning, the
subnormal range and exact cancellation, and every result must equal the
host's bit for bit.
"""
import numpy as np
import pytest

from hostcheck import hostmath as HC
from test_comp_sums import _gen_dot, _gen_pairs

pytestmark = pytest.mark.gpu


def _dot_inputs(rng, n):
    """(a, b0, b1) of shape (m, n): random, ill-conditioned, subnormal
    products, exponents over the float range, exact cancellation."""
    A, B0, B1 = [], [], []

    def add(a, b0, b1):
        A.append(np.asarray(a, np.float32))
        B0.append(np.asarray(b0, np.float32))
        B1.append(np.asarray(b1, np.float32))

    for _ in range(150):
        add(rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n))
    for _ in range(150):
        cond = float(np.exp(rng.uniform(0, np.log(1e12))))
        x, y0 = _gen_dot(rng, n, cond)
        _, y1 = _gen_dot(rng, n, cond)
        add(x, y0, y1)
    for _ in range(100):
        # products near and below the smallest normal float (2^-126)
        s = 2.0 ** rng.integers(-75, -60, 3)
        add(rng.standard_normal(n) * s[0], rng.standard_normal(n) * s[1], rng.standard_normal(n) * s[2])
    for _ in range(150):
        e = rng.integers(-70, 50, (3, n))
        add(rng.standard_normal(n) * 2.0 ** e[0], rng.standard_normal(n) * 2.0 ** e[1],
            rng.standard_normal(n) * 2.0 ** e[2])
    for _ in range(50):
        h = n // 2
        a = rng.standard_normal(h) * 2.0 ** rng.integers(-20, 20, h)
        b = rng.standard_normal(h) * 2.0 ** rng.integers(-20, 20, h)
        z = np.zeros(n - 2 * h)
        add(np.concatenate([a, a, z]), np.concatenate([b, -b, -z]), np.concatenate([-b, b, z]))
    return np.stack(A), np.stack(B0), np.stack(B1)


@pytest.mark.parametrize("levels", [2, 3])
@pytest.mark.parametrize("n", [9, 33])
def test_packed_dot_bitwise_host(levels, n):
    rng = np.random.default_rng(10 * n + levels)
    a, b0, b1 = _dot_inputs(rng, n)
    dev = HC.dev_comp_dot(levels, a, b0, b1)
    host = np.zeros_like(dev)
    for t in range(a.shape[0]):
        (h0, l0), (h1, l1) = HC.comp_dot(levels, a[t], b0[t], b1[t])
        host[t] = (h0, l0, h1, l1)
    assert np.isfinite(host).all()
    bad = np.nonzero((dev.view(np.uint32) != host.view(np.uint32)).any(axis=1))[0]
    assert bad.size == 0, (bad[:5], dev[bad[:5]], host[bad[:5]])


def _triple_inputs(rng, n):
    """(hi, lo) of shape (m, 2, n): ill-conditioned float-pair sums, pairs
    whose low halves are subnormal, zeros."""
    H, L = [], []
    for _ in range(200):
        cond = float(np.exp(rng.uniform(0, np.log(1e14))))
        h0, l0 = _gen_pairs(rng, n, cond)
        h1, l1 = _gen_pairs(rng, n, cond)
        H.append(np.stack([h0, h1]))
        L.append(np.stack([l0, l1]))
    for _ in range(100):
        h0, l0 = _gen_pairs(rng, n, 1e6)
        h1, l1 = _gen_pairs(rng, n, 1e3)
        s = np.float32(2.0 ** -118)
        H.append(np.stack([h0, h1]) * s)
        L.append(np.stack([l0, l1]) * s)
    for _ in range(20):
        H.append(np.zeros((2, n), np.float32))
        L.append(np.zeros((2, n), np.float32))
    return np.stack(H).astype(np.float32), np.stack(L).astype(np.float32)


@pytest.mark.parametrize("n", [2, 6, 12])
def test_packed_triple_sum_bitwise_host(n):
    rng = np.random.default_rng(n)
    hi, lo = _triple_inputs(rng, n)
    sub = lo[200:300]
    assert ((np.abs(sub) < np.float32(2.0 ** -126)) & (sub != 0)).any()  # subnormal low halves reached
    dev = HC.dev_triple_sum(hi, lo)
    host = np.stack([HC.triple_sum(hi[t], lo[t]) for t in range(hi.shape[0])])
    bad = np.nonzero((dev.view(np.uint64) != host.view(np.uint64)).any(axis=1))[0]
    assert bad.size == 0, (bad[:5], dev[bad[:5]], host[bad[:5]])

"""Loader of the test-only host build of the CUDA library's element math."""
import ctypes
import os
import subprocess

import numpy as np

from flexshell import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "finetoolsflexstructures.jl_gb300", "csrc")
LIB = os.path.join(HERE, "_build", "libhostcheck.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        srcs = [os.path.join(HERE, "hostcheck.cpp"), os.path.join(CSRC, "fs_elem_math.cuh"),
                os.path.join(CSRC, "fs_host_prep.h"), os.path.join(CSRC, "fs_beam_math.cuh"),
                os.path.join(CSRC, "fs_comp_sum.cuh")]
        if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
            tmp = LIB + ".tmp%d" % os.getpid()
            # no contraction of a * b + c into an FMA: the compensated sums'
            # error-free transformations need every operation rounded alone
            subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                            srcs[0], "-o", tmp], check=True)
            os.replace(tmp, LIB)
        _lib = ctypes.CDLL(LIB)
    return _lib


def element_matrices(etype, precision, xyz, conn, normals, valid, thickness, params,
                     groups=None, egroup=None):
    xyz = np.asfortranarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    normals = np.asfortranarray(normals, dtype=np.float64)
    valid = np.ascontiguousarray(valid, dtype=np.uint8)
    nelem = conn.shape[0]
    th = np.ascontiguousarray(np.broadcast_to(np.asarray(thickness, float), (nelem,)))
    nd = 6 * conn.shape[1]
    out = np.zeros((nelem, nd, nd))
    garr = None
    eg = None
    if groups is not None:
        garr = (_abi.fs_layup_group * len(groups))(*groups)
        eg = np.ascontiguousarray(egroup if egroup is not None else np.zeros(nelem), dtype=np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
    st = lib().hc_element_matrices(
        ctypes.c_int(etype), ctypes.c_int(precision), ctypes.c_int64(xyz.shape[0]), P(xyz),
        ctypes.c_int64(nelem), P(conn), P(normals), P(valid), P(th), ctypes.byref(params),
        garr, P(eg), P(out))
    if st != 0:
        raise RuntimeError("host check failed with status %d" % st)
    return out.transpose(0, 2, 1).copy()


def resultants(etype, xyz, conn, normals, valid, thickness, params, u, quantity, cs=None):
    """The library's integration-point resultant math on the host: (npoints, 3)."""
    xyz = np.asfortranarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    normals = np.asfortranarray(normals, dtype=np.float64)
    valid = np.ascontiguousarray(valid, dtype=np.uint8)
    u = np.asfortranarray(u, dtype=np.float64)
    nelem = conn.shape[0]
    th = np.ascontiguousarray(np.broadcast_to(np.asarray(thickness, float), (nelem,)))
    npt = nelem * (1 if conn.shape[1] == 3 else 4)
    if cs is None:
        ncs, csf = 0, None
    else:
        cs = np.asarray(cs, dtype=np.float64)
        ncs = 1 if cs.ndim == 2 else cs.shape[0]
        csf = np.ascontiguousarray(cs.reshape(-1, 3, 3).transpose(0, 2, 1))
    out = np.zeros((npt, 3))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
    st = lib().hc_resultants(ctypes.c_int(etype), ctypes.c_int64(xyz.shape[0]), P(xyz), ctypes.c_int64(nelem),
                             P(conn), P(normals), P(valid), P(th), ctypes.byref(params), P(u),
                             ctypes.c_int(quantity), P(csf), ctypes.c_int64(ncs), P(out))
    if st != 0:
        raise RuntimeError("host check failed with status %d" % st)
    return out


def beam_elements(which, xyz, conn, sections, E, nu, rho=0.0, u1=None, R1=None, v1=None,
                  mass_type=1, q=None):
    """The library's beam element math on the host: (nelem,12,12) or (nelem,12)."""
    xyz = np.asfortranarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    sec = np.ascontiguousarray(sections, dtype=np.float64)
    f = lambda a: None if a is None else np.asfortranarray(a, dtype=np.float64)
    u1, R1, v1 = f(u1), f(R1), f(v1)
    ne = conn.shape[0]
    if q is not None:
        q = np.ascontiguousarray(np.broadcast_to(np.asarray(q, dtype=np.float64), (ne, 3)))
    vec = which >= 4
    out = np.zeros((ne, 12 if vec else 144))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
    st = lib().hc_beam_elements(ctypes.c_int(which), ctypes.c_int64(xyz.shape[0]), P(xyz),
                                ctypes.c_int64(ne), P(conn), P(u1), P(R1), P(v1), P(sec),
                                ctypes.c_double(E), ctypes.c_double(nu), ctypes.c_double(rho),
                                ctypes.c_int(mass_type), P(q), P(out))
    assert st == 0
    return out if vec else out.reshape(ne, 12, 12).transpose(0, 2, 1).copy()


def q4_basis_pair():
    """(tabulated, computed) Q4 basis gradients at the Gauss points, 4 x 4 x 2 each."""
    out = np.zeros(64)
    lib().hc_q4_basis(out.ctypes.data_as(ctypes.c_void_p))
    return out[:32].reshape(4, 4, 2), out[32:].reshape(4, 4, 2)


def comp_dot(levels, a, b0, b1):
    """The element kernels' compensated dot products (a . b0, a . b1) of float
    vectors at 2 (Dot2) or 3 levels: ((hi0, lo0), (hi1, lo1)) as float32."""
    a, b0, b1 = (np.ascontiguousarray(v, dtype=np.float32) for v in (a, b0, b1))
    out = np.zeros(4, dtype=np.float32)
    P = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    st = lib().hc_comp_dot(ctypes.c_int(levels), ctypes.c_int(a.size), P(a), P(b0), P(b1), P(out))
    assert st == 0
    return (out[0], out[1]), (out[2], out[3])


def triple_sum(hi, lo):
    """The gather's column sums of float pairs: hi, lo of shape (2, n), one
    column per f32x2 lane; returns the two sums rounded to double."""
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    assert hi.shape == lo.shape and hi.shape[0] == 2
    out = np.zeros(2)
    P = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    st = lib().hc_triple_sum(ctypes.c_int(hi.shape[1]), P(hi), P(lo), P(out))
    assert st == 0
    return out


DEVLIB = os.path.join(HERE, "_build", "libdevcheck.so")
_devlib = None


def dev_lib():
    """The test-only device build of the compensated sums (devcheck.cu), for
    sm_103a; needs nvcc and a GPU."""
    global _devlib
    if _devlib is None:
        os.makedirs(os.path.dirname(DEVLIB), exist_ok=True)
        srcs = [os.path.join(HERE, "devcheck.cu"), os.path.join(CSRC, "fs_comp_sum.cuh")]
        if not os.path.exists(DEVLIB) or any(os.path.getmtime(s) > os.path.getmtime(DEVLIB) for s in srcs):
            from flexshell import build as B
            tmp = DEVLIB + ".tmp%d" % os.getpid()
            subprocess.run([B.nvcc()] + B.ARCH + ["-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                                                  "-I", CSRC, srcs[0], "-o", tmp], check=True)
            os.replace(tmp, DEVLIB)
        _devlib = ctypes.CDLL(DEVLIB)
    return _devlib


def dev_comp_dot(levels, a, b0, b1):
    """comp_dot on the GPU for m inputs at once: a, b0, b1 of shape (m, n);
    returns (m, 4) float32: hi0, lo0, hi1, lo1."""
    a, b0, b1 = (np.ascontiguousarray(v, dtype=np.float32) for v in (a, b0, b1))
    m, n = a.shape
    assert b0.shape == (m, n) and b1.shape == (m, n)
    out = np.zeros((m, 4), dtype=np.float32)
    P = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    st = dev_lib().dc_comp_dot(ctypes.c_int(levels), ctypes.c_int(n), ctypes.c_int(m), P(a), P(b0), P(b1), P(out))
    assert st == 0, st
    return out


def dev_triple_sum(hi, lo):
    """triple_sum on the GPU for m inputs at once: hi, lo of shape (m, 2, n);
    returns (m, 2) doubles."""
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    m, two, n = hi.shape
    assert two == 2 and lo.shape == hi.shape
    out = np.zeros((m, 2))
    P = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    st = dev_lib().dc_triple_sum(ctypes.c_int(n), ctypes.c_int(m), P(hi), P(lo), P(out))
    assert st == 0, st
    return out

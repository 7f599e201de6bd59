"""Writes raasch_hook.npz: the four Raasch hook meshes of the reference's
test-suite (test/raasch_s4_1x9.inp, _3x18, _5x36, _10x72; read by
test/test_shell_statics.jl:143-227 through FinEtools' import_ABAQUS), the
LE5 Z-section cantilever (test/nle5xf3c.inp, :441-531) and the irregular
barrel vault (test/barrelvault_stri3_irreg.inp, :578-758) as plain arrays, so
that the tests run where the reference is absent.

For each mesh the S4 quadrilaterals (S3R or STRI3 triangles) and
the coordinates of the nodes they use are kept, with the nodes renumbered in
their file order (findunconnnodes + compactnodes of the reference tests); the
split into triangles (Q4toT3) is left to the tests.  Run from the repository
root with the reference's test directory as the one argument:

    python tests/golden/make_raasch_hook.py <reference>/test
"""
import os
import sys

import numpy as np

MESHES = ["1x9", "3x18", "5x36", "10x72"]


def read_abaqus_s4(path, etype="s4", nen=4):
    """Node coordinates and the connectivity of one shell element type
    (S4: 4 nodes, S3R: 3 nodes) of the first part of an Abaqus input file
    (the data lines after *Node and *Element, type=...)."""
    nodes, elems, mode = {}, [], None
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("**"):
                continue
            if s.startswith("*"):
                kw = s.lower().replace(" ", "")
                if kw.startswith("*node") and not kw.startswith("*nodeoutput"):
                    mode = "node" if not nodes else None
                elif kw.startswith("*element,") and kw.split("type=")[-1].split(",")[0] == etype:
                    mode = "elem"
                else:
                    mode = None
                continue
            v = [t for t in s.split(",") if t.strip()]
            if mode == "node":
                nodes[int(v[0])] = [float(t) for t in v[1:4]]
            elif mode == "elem":
                elems.append([int(t) for t in v[1:1 + nen]])
    ids = np.array(sorted(nodes))
    xyz = np.array([nodes[i] for i in ids], dtype=np.float64)
    conn = np.array(elems, dtype=np.int64)
    # compact: keep the connected nodes in their order, renumber 1-based
    used = np.zeros(ids.max() + 1, dtype=bool)
    used[conn.ravel()] = True
    keep = used[ids]
    newnum = np.zeros(ids.max() + 1, dtype=np.int64)
    newnum[ids[keep]] = np.arange(1, keep.sum() + 1)
    return xyz[keep], newnum[conn]


def main(src):
    out = {}
    for m in MESHES:
        xyz, conn = read_abaqus_s4(os.path.join(src, "raasch_s4_%s.inp" % m))
        out["xyz_" + m] = xyz
        out["conn_" + m] = conn
        print(m, xyz.shape[0], "nodes", conn.shape[0], "quads")
    xyz, conn = read_abaqus_s4(os.path.join(src, "nle5xf3c.inp"), "s3r", 3)
    out["xyz_le5"] = xyz
    out["conn_le5"] = conn
    print("le5", xyz.shape[0], "nodes", conn.shape[0], "triangles")
    xyz, conn = read_abaqus_s4(os.path.join(src, "barrelvault_stri3_irreg.inp"), "stri3", 3)
    out["xyz_vault"] = xyz
    out["conn_vault"] = conn
    print("vault", xyz.shape[0], "nodes", conn.shape[0], "triangles")
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "raasch_hook.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_raasch_hook.py <reference test directory>")
    main(sys.argv[1])

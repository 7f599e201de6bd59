"""The oracle's pattern-accumulating check helper (orc_csc_accumulate_stiffness,
used for meshes too large for its COO assembly) against its own COO assembly."""
import numpy as np
import pytest

from oracle import oracle as O
from flexshell import materials
import problems as PB


@pytest.mark.parametrize("quads", [False, True])
def test_into_pattern_equals_coo_assembly(quads):
    xyz, conn, dof, nfree = PB.jittered_plate(10, quads, wavy=0.01, seed=4)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(200e9, 0.3, 7850.0))
    P = O.Problem(O.Q4RS if quads else O.T3FF, xyz, conn, dof, thickness=0.005,
                  material=dict(Dps=Dps, Dt=Dt, rho=7850.0))
    P.compute_normals()
    for n in (int(dof.max()), nfree):
        colptr, rowval, nzval, _ = P.assemble("K", O.KEEP_ZEROS, n=n)
        vals, touched, missing = P.stiffness_into_pattern(colptr, rowval, n=n)
        assert missing == 0 and touched.all()
        assert np.abs(vals - nzval).max() <= 1e-14 * np.abs(nzval).max()
        # a pattern without one stored entry: its contributions are counted as missing
        k = len(rowval) // 2
        col = np.searchsorted(colptr - 1, k, side="right") - 1
        cp2 = colptr.copy()
        cp2[col + 1:] -= 1
        rv2 = np.delete(rowval, k)
        _, t2, miss2 = P.stiffness_into_pattern(cp2, rv2, n=n)
        assert miss2 > 0 and t2.all()

"""GPU nodal normals with a built-in material csys (fs_normals_compute_csys)
against the oracle: normals within 1e-14, identical validity flags, and the
stiffness assembled with them within 1e-12."""
import numpy as np
import pytest

import flexshell as F
from flexshell import _abi
from flexshell._lib import FlexShellError, ptr
from oracle import oracle as O
from checks import relmax, same_pattern
from test_csys_normals import MAT, cylinder_panel, flat_plate
from test_gpu_parity import _Mat

pytestmark = pytest.mark.gpu

KINDS = [
    ("cylindrical", F.CSysCylindrical([0.0, 0.0, 0.0], [0.0, 1.0, 0.0]), O.CSYS_CYLINDRICAL, [0, 0, 0, 0, 1, 0]),
    ("spherical", F.CSysSpherical([0.3, 1.0, -0.5]), O.CSYS_SPHERICAL, [0.3, 1.0, -0.5]),
    ("cartesian", F.CSysCartesian(np.column_stack([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])),
     O.CSYS_CARTESIAN, np.column_stack([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])),
]


@pytest.mark.parametrize("quads", [False, True])
@pytest.mark.parametrize("kind", KINDS, ids=[k[0] for k in KINDS])
def test_csys_normals_match_oracle(quads, kind):
    name, cs, okind, oprm = kind
    xyz, conn = cylinder_panel(quads) if name != "cartesian" else flat_plate(quads)
    f = F.NodalField(np.zeros((xyz.shape[0], 6)))
    f.numberdofs()
    et = O.Q4RS if quads else O.T3FF
    P = O.Problem(et, xyz, conn, f.dofnums, thickness=0.01, material=MAT)
    nrm, val = P.compute_normals(30.0, okind, oprm)
    cls = F.FEMMShellQ4RS if quads else F.FEMMShellT3FF
    femm = cls(conn, 0.01, _Mat(MAT), mcsys=cs)
    geom0 = F.NodalField(xyz)
    femm.associategeometry(geom0)
    assert np.abs(femm._normals - nrm).max() <= 1e-14
    assert np.array_equal(femm._normal_valid, val)
    K = femm.stiffness(F.SysmatAssemblerSparse(), geom0, None, None, f)
    Ko = P.assemble_scipy("K", O.KEEP_ZEROS)
    assert same_pattern(K, Ko) and relmax(K, Ko) <= 1e-12
    femm.close()


def test_csys_errors():
    xyz, conn = flat_plate(False)
    femm = F.FEMMShellT3FF(conn, 0.01, _Mat(MAT))
    femm._upload_mesh(F.NodalField(xyz))
    with pytest.raises(FlexShellError) as ei:
        femm.ctx.call("fs_normals_compute_csys", 9, ptr(np.zeros(9)))
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    with pytest.raises(FlexShellError) as ei:
        femm.ctx.call("fs_normals_compute_csys", _abi.FS_CSYS_SPHERICAL, None)
    assert ei.value.code == _abi.FS_ERR_BAD_INPUT
    femm.close()

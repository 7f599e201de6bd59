"""ctypes mirror of include/flexshell.h (structs and constants)."""
import ctypes

FS_OK = 0
FS_ERR_BAD_INPUT = 1
FS_ERR_CUDA = 2
FS_ERR_OOM = 3
FS_ERR_SINGULAR_METRIC = 4
FS_ERR_UNSUPPORTED = 5
FS_ERR_STATE = 6
FS_ERR_TIMEOUT = 7

FS_T3FF, FS_T3FFCOMP, FS_Q4RS, FS_Q4RSCOMP, FS_COROTBEAM = 0, 1, 2, 3, 4
FS_FP64, FS_MIXED, FS_MIXED_COMP = 0, 1, 2
FS_ASM_SPARSE, FS_ASM_SPARSE_SYMM, FS_ASM_DIAG = 0, 1, 2
FS_BEAM_STIFFNESS, FS_BEAM_GEOSTIFFNESS, FS_BEAM_MASS, FS_BEAM_GYROSCOPIC = 0, 1, 2, 3
FS_BEAM_RESTORING, FS_BEAM_DISTRIBLOAD = 4, 5
FS_RES_MOMENT, FS_RES_SHEAR, FS_RES_MEMBRANE = 1, 2, 3
FS_CSYS_ISOPARAMETRIC, FS_CSYS_CARTESIAN, FS_CSYS_CYLINDRICAL, FS_CSYS_SPHERICAL = 0, 1, 2, 3


class fs_beam_section(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("A", "I1", "I2", "I3", "J", "A2s", "A3s")] + [
        ("x1x2_vector", ctypes.c_double * 3)]


class fs_shell_params(ctypes.Structure):
    _fields_ = [
        ("transv_shear_formulation", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("drilling_stiffness_scale", ctypes.c_double),
        ("threshold_angle", ctypes.c_double),
        ("stab_c", ctypes.c_double),
        ("Dps", ctypes.c_double * 9),
        ("Dt", ctypes.c_double * 4),
        ("rho", ctypes.c_double),
        ("thickness", ctypes.c_double),
    ]


class fs_layup_group(ctypes.Structure):
    _fields_ = [
        ("A", ctypes.c_double * 9),
        ("B", ctypes.c_double * 9),
        ("D", ctypes.c_double * 9),
        ("H", ctypes.c_double * 4),
        ("csmat", ctypes.c_double * 9),
        ("thickness", ctypes.c_double),
        ("mass_density", ctypes.c_double),
        ("moi_density", ctypes.c_double),
    ]


def _colmajor(a, n):
    import numpy as np
    v = np.asarray(a, dtype=np.float64).flatten(order="F")
    assert v.size == n
    return list(v)


def make_params(Dps, Dt, rho=0.0, thickness=0.0, stab_c=None, drilling_stiffness_scale=1.0,
                threshold_angle=30.0, transv_shear_formulation=0, quads=False):
    p = fs_shell_params()
    p.transv_shear_formulation = transv_shear_formulation
    p.drilling_stiffness_scale = drilling_stiffness_scale
    p.threshold_angle = threshold_angle
    if stab_c is None:
        stab_c = 0.1 if quads else 5 / 12 / 1.5
    p.stab_c = stab_c
    p.Dps[:] = _colmajor(Dps, 9)
    p.Dt[:] = _colmajor(Dt, 4)
    p.rho = rho
    p.thickness = thickness
    return p


def make_group(A, B, D, H, csmat, thickness, mass_density=0.0, moi_density=0.0):
    g = fs_layup_group()
    g.A[:] = _colmajor(A, 9)
    g.B[:] = _colmajor(B, 9)
    g.D[:] = _colmajor(D, 9)
    g.H[:] = _colmajor(H, 4)
    g.csmat[:] = _colmajor(csmat, 9)
    g.thickness = thickness
    g.mass_density = mass_density
    g.moi_density = moi_density
    return g

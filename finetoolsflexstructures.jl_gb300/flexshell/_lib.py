"""ctypes binding of libflexshell.so (the C ABI of include/flexshell.h).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every call raises; nothing falls back to the CPU.
"""
import ctypes
import os

import numpy as np

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libflexshell.so")

_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)

_lib = None


class FlexShellError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("flexshell error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libflexshell.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        from . import build as _build
        _build.build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.fs_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.fs_ctx_destroy.argtypes = [vp]
        L.fs_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
        L.fs_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.fs_mesh_set.argtypes = [vp, ctypes.c_int, ctypes.c_int64, vp, ctypes.c_int64, vp, vp, vp]
        L.fs_params_set.argtypes = [vp, ctypes.POINTER(_abi.fs_shell_params), vp]
        L.fs_layups_set.argtypes = [vp, ctypes.c_int32, vp, vp]
        L.fs_normals_compute.argtypes = [vp]
        L.fs_normals_set.argtypes = [vp, vp, vp]
        L.fs_normals_get.argtypes = [vp, vp, vp]
        L.fs_stiffness.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _c_i64_p]
        L.fs_mass.argtypes = [vp, ctypes.c_int, ctypes.c_int64, _c_i64_p]
        L.fs_matrix_copy.argtypes = [vp, vp, vp, vp]
        L.fs_matrix_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                       _c_i64_p, _c_i64_p]
        L.fs_element_matrices.argtypes = [vp, ctypes.c_int, vp]
        L.fs_timings.argtypes = [vp, vp, ctypes.c_int]
        L.fs_stiffness_values_noalloc.argtypes = [vp, ctypes.c_int, ctypes.c_int64, vp, ctypes.c_int64]
        L.fs_geometry_set.argtypes = [vp, vp]
        L.fs_dofs_set.argtypes = [vp, vp]
        L.fs_element_masses.argtypes = [vp, vp]
        L.fs_explicit_setup.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_double]
        L.fs_explicit_set_state.argtypes = [vp, vp, vp, vp]
        L.fs_explicit_run.argtypes = [vp, ctypes.c_int64]
        L.fs_explicit_set_load.argtypes = [vp, vp, vp, ctypes.c_int64, ctypes.c_int64]
        L.fs_explicit_get_state.argtypes = [vp, vp, vp, vp]
        L.fs_power_iteration.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_uint64, vp]
        L.fs_laminate.argtypes = [ctypes.c_int32, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_int32,
                                  ctypes.c_double, ctypes.POINTER(_abi.fs_layup_group)]
        L.fs_restoring_force.argtypes = [vp, vp, vp]
        L.fs_resultants.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int64, vp]
        L.fs_distribloads.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64, vp]
        L.fs_integration_points.argtypes = [vp, ctypes.c_int, vp]
        L.fs_normals_compute_csys.argtypes = [vp, ctypes.c_int, vp]
        L.fs_pattern.argtypes = [vp, ctypes.c_int64, _c_i64_p]
        L.fs_stiffness_copy.argtypes = [vp, ctypes.c_int, ctypes.c_int64, vp, vp, vp]
        L.fs_autotune.argtypes = [vp, ctypes.c_int]
        L.fs_tuning.argtypes = [vp, vp]
        L.fs_tuning_ex.argtypes = [vp, vp, ctypes.c_int]
        L.fs_batch_set.argtypes = [vp, ctypes.c_int, ctypes.c_int32, vp, vp, vp, vp, vp, vp, vp]
        L.fs_batch_stiffness.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.fs_batch_matrix_copy.argtypes = [vp, ctypes.c_int32, vp, vp, vp]
        L.fs_beam_setup.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.fs_beam_state_set.argtypes = [vp, vp, vp, vp]
        L.fs_beam_matrix.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, _c_i64_p]
        L.fs_beam_restoringforce.argtypes = [vp, ctypes.c_int64, vp]
        L.fs_beam_distribloads_global.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int64, vp]
        L.fs_beam_element_matrices.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        L.fs_beam_element_vectors.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp]
        L.fs_shift_factor.argtypes = [vp, ctypes.c_double, vp, _c_i64_p]
        L.fs_shift_solve.argtypes = [vp, ctypes.c_int, vp, vp]
        _lib = L
    return _lib


class InputCache:
    """A host copy of the array last uploaded to a context.  The reference
    reads geom0 and dchi on every call, so an upload is repeated exactly when
    the caller's array differs from the copy: replaced or changed in place
    (an identity key would miss both an in-place change and a new array that
    reuses a freed one's address)."""

    def __init__(self):
        self.copy = None

    def stale(self, a):
        return self.copy is None or self.copy.shape != a.shape or not np.array_equal(self.copy, a)

    def store(self, a):
        self.copy = np.array(a, copy=True, order="F")

    def clear(self):
        self.copy = None


def ptr(a):
    """Address of a numpy array (or None)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """One library context (device memory, stream) on one GPU."""

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        st = lib().fs_ctx_create(device, ctypes.byref(self._h))
        if st != 0:
            raise FlexShellError(st, "cannot create a context on CUDA device %d" % device)

    @property
    def handle(self):
        return self._h

    def check(self, st):
        if st != 0:
            buf = ctypes.create_string_buffer(512)
            lib().fs_last_error(self._h, buf, 512)
            raise FlexShellError(st, buf.value.decode(errors="replace"))

    def call(self, name, *args):
        self.check(getattr(lib(), name)(self._h, *args))

    def stream(self):
        s = ctypes.c_void_p()
        self.check(lib().fs_stream(self._h, ctypes.byref(s)))
        return s.value

    def close(self):
        if self._h and self._h.value:
            lib().fs_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def laminate(plies, offset=0.0, shear_model=0, tcf=0.0):
    """Layup reduction with the library (fs_laminate): returns an fs_layup_group."""
    k = len(plies)
    Dps = np.ascontiguousarray(np.concatenate([np.asarray(p["Dps"], float).flatten(order="F") for p in plies]))
    Dts = np.ascontiguousarray(np.concatenate([np.asarray(p["Dts"], float).flatten(order="F") for p in plies]))
    t = np.ascontiguousarray([p["thickness"] for p in plies], dtype=np.float64)
    ang = np.ascontiguousarray([p["angle"] for p in plies], dtype=np.float64)
    rho = np.ascontiguousarray([p.get("rho", 0.0) for p in plies], dtype=np.float64)
    g = _abi.fs_layup_group()
    st = lib().fs_laminate(k, ptr(Dps), ptr(Dts), ptr(t), ptr(ang), ptr(rho), offset, shear_model, tcf,
                           ctypes.byref(g))
    if st != 0:
        raise FlexShellError(st, "invalid layup")
    return g

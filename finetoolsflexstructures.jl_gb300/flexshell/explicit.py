"""Central-difference time stepping on the GPU: the `_cd_loop!` of the
reference's explicit examples
(examples/shells/dynamics/homogeneous/explicit/plate_expl_examples.jl:61-94).

The stiffness is the last one assembled by the FEMM's context (it stays on
the device); mass-proportional damping and the example's external force
force!(F, t) = g(t) Fmag run inside the captured step loop (fs_explicit_*).
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import ptr


class CentralDifference:
    """The step loop of one stiffness: M the diagonal mass (vector), C the
    damping (vector), dt the time step; precision FS_FP64, FS_MIXED (float
    restoring force, double state) or FS_MIXED_COMP (float values, the
    restoring force summed in compensated float sums from a float-pair copy
    of U)."""

    def __init__(self, femm, M, C, dt, precision=_abi.FS_FP64):
        self.ctx = femm.ctx
        self.n = int(np.asarray(M).shape[0])
        self.dt = float(dt)
        m = np.ascontiguousarray(M, dtype=np.float64)
        self.C = np.ascontiguousarray(C, dtype=np.float64)
        self.invMC = np.ascontiguousarray(1.0 / (m + (self.dt / 2) * self.C))
        self.ctx.call("fs_explicit_setup", precision, ptr(self.invMC), ptr(self.C), ctypes.c_double(self.dt))
        self._load = None

    def set_state(self, U, V, A):
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (U, V, A)]
        self.ctx.call("fs_explicit_set_state", *[ptr(a) for a in arr])

    def set_load(self, Fmag, g, nsteps, step0=0):
        """F(t) = g(t) Fmag; g a callable of t or the values g(k dt) for k = 0..
        (evaluated at k = 0..step0 + nsteps when callable).  Fmag None: no load."""
        if Fmag is None:
            self._load = None
            self.ctx.call("fs_explicit_set_load", None, None, 0, 0)
            return
        Fm = np.ascontiguousarray(Fmag, dtype=np.float64)
        if callable(g):
            mul = np.array([g(k * self.dt) for k in range(step0 + nsteps + 1)], dtype=np.float64)
        else:
            mul = np.ascontiguousarray(g, dtype=np.float64)
        self._load = (Fm, mul)
        self.ctx.call("fs_explicit_set_load", ptr(Fm), ptr(mul), mul.shape[0], step0)

    def run(self, nsteps):
        self.ctx.call("fs_explicit_run", int(nsteps))

    def state(self):
        U, V, A = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        self.ctx.call("fs_explicit_get_state", ptr(U), ptr(V), ptr(A))
        return U, V, A


def cd_loop(femm, M, ksi, omegad, U0, V0, tend, dt, Fmag=None, g=None, peek=None, peek_every=1,
            precision=_abi.FS_FP64):
    """_cd_loop!(M, K, ksi, U0, V0, tend, dt, force!, peek) with K the FEMM's
    last stiffness, C = ksi 2 omegad diag(M), and force!(F, t) = g(t) Fmag (no
    load when Fmag is None).  The time step is adjusted as in the reference
    (nsteps = round(tend/dt); if nsteps dt < tend, dt = tend/(nsteps + 1)).
    peek(step, U, V, t) is called at step 0 and after every peek_every steps
    (the state is copied to the host for it).  Returns the final U, V, A."""
    m = np.asarray(M if np.ndim(M) == 1 else M.diagonal(), dtype=np.float64)
    C = (ksi * 2 * omegad) * m
    nsteps = int(round(tend / dt))
    if nsteps * dt < tend:
        dt = tend / (nsteps + 1)
    cd = CentralDifference(femm, m, C, dt, precision)
    mul = None
    A0 = np.zeros(m.shape[0])
    if Fmag is not None:
        mul = np.array([g(k * dt) for k in range(nsteps + 1)], dtype=np.float64) if callable(g) \
            else np.asarray(g, dtype=np.float64)
        A0 = cd.invMC * (mul[0] * np.asarray(Fmag, dtype=np.float64))
    cd.set_state(U0, V0, A0)
    if Fmag is not None:
        cd.set_load(Fmag, mul, nsteps)
    if peek is not None:
        peek(0, np.asarray(U0, dtype=np.float64).copy(), np.asarray(V0, dtype=np.float64).copy(), 0.0)
    done = 0
    every = max(int(peek_every), 1) if peek is not None else nsteps
    while done < nsteps:
        k = min(every, nsteps - done)
        cd.run(k)
        done += k
        if peek is not None:
            U, V, _ = cd.state()
            peek(done, U, V, done * dt)
    return cd.state()

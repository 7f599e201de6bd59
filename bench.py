"""Benchmark of the shell element-assembly hot path on one GB300.

Workload (the reference's configuration 2, synthetic): a 1024 x 1024 quad
plate on [0,1]^2, interior nodes jittered U(+-0.2 h) (PCG64 seed 0),
z = 0.01 sin(pi x) sin(pi y), thickness 0.005, steel (E 200 GPa, nu 0.3,
rho 7850).  T3FF uses the 2,097,152 triangles of the split quads, Q4RS the
1,048,576 quads; 1,050,625 nodes x 6 dofs, all dofs in the matrix.

A step is one stiffness assembly: element matrices + deterministic CSR value
gather, on device-resident inputs with the sparsity pattern built (it depends
only on the mesh and is built once per mesh; its time is reported apart).
`value` is T3FF elements assembled per second in the compensated mixed mode
(FS_MIXED_COMP: float element rows, Gram products accumulated in compensated
sums and kept as float pairs, double CSR values), the mode whose stiffness, mass and
20 lowest layered-plate eigenvalues are all within 1e-6 of FP64; the plain
mixed mode (FS_MIXED), the FP64 path and Q4RS are reported beside it.  `e2e`
is the same assembly through the C ABI from pinned host buffers: geometry and
dof numbering uploaded, pattern rebuilt, assembled, CSC arrays (colptr,
rowval, nzval) copied back.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "finetoolsflexstructures.jl_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

METRIC = "shell elements assembled/s, mixed vs FP64 on one GB300 at <=1e-6 rel err; CPU ref"
E, NU, RHO, THICK = 200e9, 0.3, 7850.0, 0.005


def plate(n, quads, seed=0):
    from flexshell import mesh
    xyz, connq = mesh.jittered_plate_q(n, 1.0, 0.2, seed,
                                       lambda x, y: 0.01 * np.sin(np.pi * x) * np.sin(np.pi * y))
    conn = connq if quads else mesh.quads_to_triangles(connq)
    dof, nfree = mesh.numberdofs(np.zeros((xyz.shape[0], 6), bool))
    return np.asfortranarray(xyz), np.ascontiguousarray(conn), np.asfortranarray(dof)


def params(quads):
    from flexshell import _abi, materials
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, NU, RHO))
    return _abi.make_params(Dps, Dt, RHO, THICK, quads=quads)


# DRAM bytes (read + write) per element of one launch of each kernel of the
# T3FF step, from ncu captures of the 512 x 512 plate (524,288 triangles; the
# full-size launch is beyond the capture size rule): dram__bytes_read.sum +
# dram__bytes_write.sum divided by the elements of the launch.  Source: the
# capture named beside each figure (its summary and command are committed
# under profiles/); the figures are scaled to the benchmark's element count,
# traffic growing in proportion to the elements at a fixed mesh type.
MEASURED_TRAFFIC_PER_ELEMENT = {
    "k_t3_elements FS_MIXED": (802.2, "ncu --set full, k_t3_elements, FS_MIXED, T3FF 512^2 "
                                      "(profiles/k_t3_elements_k_gather_t3ff_mixed_512.md)"),
    "k_gather FS_MIXED": (1983.5, "ncu --set full, k_gather, FS_MIXED, T3FF 512^2 "
                                  "(profiles/k_t3_elements_k_gather_t3ff_mixed_512.md)"),
    "k_t3_elements FS_MIXED_COMP": (1668.8, "ncu --set full, k_t3_elements, FS_MIXED_COMP, T3FF 512^2 "
                                            "(profiles/k_t3_elements_k_gather_t3ff_mixed_comp_512.md)"),
    "k_gather FS_MIXED_COMP": (2874.2, "ncu --set full, k_gather, FS_MIXED_COMP, T3FF 512^2 "
                                       "(profiles/k_t3_elements_k_gather_t3ff_mixed_comp_512.md)"),
}


def measured_traffic(kernel, nelem):
    """DRAM bytes of one launch of `kernel` over `nelem` elements from the
    per-element ncu figure above, and its source; (None, None) when the
    kernel has not been captured."""
    if kernel not in MEASURED_TRAFFIC_PER_ELEMENT:
        return None, None
    per, src = MEASURED_TRAFFIC_PER_ELEMENT[kernel]
    return per * nelem, src


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during a timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # the sampler's start-up, so that it covers the region that follows
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p is not None:
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if len(f) > 2 + k and f[2 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(steps=1, warmup=0, n=1024, nthreads=None):
    """The oracle (C restatement of the reference's stiffness loop and of
    FinEtools' COO -> sparse(I, J, V) assembly; the element loop over OpenMP
    threads, the assembly serial as Julia's sparse) on the n x n plate of the
    workload's construction (seed 0, jitter, wave, thickness, steel) split in
    triangles: n = 1024 is the workload itself.  warmup untimed steps, then
    `steps` timed ones; nthreads None: every host core."""
    from oracle import oracle as O
    from flexshell import materials
    xyz, conn, dof = plate(n, False)
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, NU, RHO))
    P = O.Problem(O.T3FF, xyz, conn, dof, thickness=THICK, material=dict(Dps=Dps, Dt=Dt, rho=RHO))
    P.compute_normals()
    cores = nthreads or os.cpu_count() or 1
    for _ in range(warmup):
        P.assemble("K", O.KEEP_ZEROS, nthreads=cores)
    times = []
    for _ in range(max(steps, 1)):
        t1 = time.perf_counter()
        P.assemble("K", O.KEEP_ZEROS, nthreads=cores)
        times.append(time.perf_counter() - t1)
    el = conn.shape[0]
    what = ("the full %dx%d workload (%d triangles)" % (n, n, el) if n == 1024 else
            "a %dx%d plate of the workload's construction (%d triangles, 1/%d of the 1024x1024 workload)"
            % (n, n, el, (1024 // n) ** 2))
    return {"value": el * len(times) / sum(times), "unit": "elements/s", "cores": cores, "kind": "port",
            "sample": "T3FF stiffness, %s, element loop + COO->CSC assembly, %d timed step(s) after %d "
                      "untimed" % (what, len(times), warmup)}, times


def cpu_sample_side(nsteps, budget_s=200.0, nthreads=None):
    """The largest plate side (1024, the workload, then 512, 256, 128) whose
    nsteps oracle steps fit `budget_s` seconds, from one timed 128 x 128 step
    scaled by the element count (the assembly is close to linear in it)."""
    _, t = cpu_baseline(steps=1, n=128, nthreads=nthreads)
    for n in (1024, 512, 256):
        if nsteps * t[0] * (n / 128) ** 2 * 1.2 <= budget_s:
            return n
    return 128


def max_over_ranks(x, world, dist):
    """The largest value over the ranks (the slowest replica's time); x itself
    on one rank.  NCCL reduces a device tensor, gloo a host one."""
    if world <= 1:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_text(n):
    nodes = (n + 1) ** 2
    return "T3FF stiffness assembly, %dx%d jittered wavy plate (%d triangles, %d nodes, %d dofs)" % (
        n, n, 2 * n * n, nodes, 6 * nodes)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    # the workload itself when its warm-up and timed steps fit a few minutes
    n = cpu_sample_side(args.warmup + args.steps)
    cb, times = cpu_baseline(steps=args.steps, warmup=max(args.warmup, 1), n=n)
    ms = 1e3 * float(np.mean(times))
    line = {"metric": METRIC, "value": cb["value"], "unit": "elements/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload_text(args.n), "precision": "FP64 (the reference's arithmetic)",
                       "sample": cb["sample"], "same_workload": n == args.n},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def oracle_check_c2(asm, xyz, conn, dof, quads, nnz):
    """FP64 stiffness of the full-size plate against the oracle (outside every
    timed region): the oracle's element matrices (the reference's loop) are
    summed into the GPU matrix's own pattern, which also checks the pattern
    (no oracle contribution outside it, every stored entry reached), and
    compared entrywise; the lumped mass diagonal likewise."""
    from oracle import oracle as O
    from flexshell import _abi, materials
    n = asm.n
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, NU, RHO))
    P = O.Problem(O.Q4RS if quads else O.T3FF, xyz, conn, dof, thickness=THICK,
                  material=dict(Dps=Dps, Dt=Dt, rho=RHO))
    P.compute_normals()
    t0 = time.perf_counter()
    asm.stiffness(_abi.FS_FP64)
    colptr = np.empty(n + 1, dtype=np.int64)
    rowval = np.empty(nnz, dtype=np.int64)
    v = np.empty(nnz)
    asm.ctx.call("fs_matrix_copy", asm.ptr(colptr), asm.ptr(rowval), asm.ptr(v))
    vo, touched, missing = P.stiffness_into_pattern(colptr, rowval, n=n)
    # entrywise measures (as tests/checks.entrywise_errors), on the shared pattern
    d = np.zeros(n)
    cols = np.repeat(np.arange(n), np.diff(colptr))
    diag = rowval - 1 == cols
    d[cols[diag]] = np.abs(vo[diag])
    dv = np.abs(v - vo)
    mx = np.abs(vo).max()
    den = np.sqrt(d[rowval - 1] * d[cols])
    ok = den > 0
    big = np.abs(vo) > 1e-12 * mx
    out = {"elements": int(conn.shape[0]), "pattern_identical": bool(missing == 0 and touched.all()),
           "rel_err_K_fp64_vs_oracle_max": float(dv.max() / mx),
           "rel_err_K_fp64_vs_oracle_scaled": float((dv[ok] / den[ok]).max()),
           "rel_err_K_fp64_vs_oracle_entrywise": float((dv[big] / np.abs(vo[big])).max()),
           "entrywise_floor": "entries above 1e-12 max|K|; scaled: |dK_ij| / sqrt(|K_ii K_jj|)"}
    del colptr, rowval, v, vo, touched, cols, diag, dv, den, ok, big
    nnzd = ctypes.c_int64()
    asm.ctx.call("fs_mass", _abi.FS_ASM_DIAG, ctypes.c_int64(n), ctypes.byref(nnzd))
    m = np.empty(n)
    asm.ctx.call("fs_matrix_copy", None, None, asm.ptr(m))
    _, _, mo, _ = P.assemble("M", O.DIAG, n=n)
    out["rel_err_M_fp64_vs_oracle_max"] = float(np.abs(m - mo).max() / np.abs(mo).max())
    out["seconds"] = time.perf_counter() - t0
    return out


class Assembler:
    """One library context with one mesh resident."""

    def __init__(self, xyz, conn, dof, quads, device=0):
        from flexshell import _abi
        from flexshell._lib import Context, ptr
        self.ptr = ptr
        self.ctx = Context(device)
        self.quads = quads
        self.nelem = conn.shape[0]
        self.n = dof.shape[0] * 6
        et = _abi.FS_Q4RS if quads else _abi.FS_T3FF
        self.ctx.call("fs_mesh_set", et, xyz.shape[0], ptr(xyz), conn.shape[0], ptr(conn), None, ptr(dof))
        self.ctx.call("fs_params_set", params(quads), None)
        self.ctx.call("fs_normals_compute")

    def stiffness(self, precision):
        nnz = ctypes.c_int64()
        self.ctx.call("fs_stiffness", precision, 0, self.n, ctypes.byref(nnz))
        return nnz.value

    def tiles(self):
        t = (ctypes.c_int32 * 4)()
        self.ctx.call("fs_tuning_ex", t, 4)
        return {"elements_per_block": t[0], "gather_warps": t[1], "tuned": bool(t[2]), "pairs_once": bool(t[3])}

    def timings(self):
        t = np.zeros(4)
        self.ctx.call("fs_timings", self.ptr(t), 4)
        return t

    def values(self, nnz):
        v = np.empty(nnz)
        self.ctx.call("fs_matrix_copy", None, None, self.ptr(v))
        return v


def explicit_c5(torch, device=0, n=512, nsteps=10000, iters=200):
    """Explicit dynamics (the reference's configuration 5): Q4RS 512 x 512 plate,
    t = 0.01, steel, simply supported (w = 0 on the boundary), lumped mass,
    V0_z = 1e-3 sin(pi x) sin(pi y) + N(0, 1e-5) (seed 5), no damping,
    dt = 0.9 * 2 / omega_max (power iteration), 10,000 steps, stiffness values
    in float (mixed) and double, state in double with Kahan compensation."""
    from flexshell import _abi, mesh
    from flexshell._lib import Context, ptr
    xyz, conn = mesh.jittered_plate_q(n, 1.0, 0.0, 0, None)
    xyz = np.asfortranarray(xyz)
    fixed = np.zeros((xyz.shape[0], 6), bool)
    x, y = xyz[:, 0], xyz[:, 1]
    bnd = (x < 1e-12) | (x > 1 - 1e-12) | (y < 1e-12) | (y > 1 - 1e-12)
    fixed[bnd, 2] = True
    dof, nfree = mesh.numberdofs(fixed)
    dof = np.asfortranarray(dof)
    ctx = Context(device)
    ctx.call("fs_mesh_set", _abi.FS_Q4RS, xyz.shape[0], ptr(xyz), conn.shape[0], ptr(np.ascontiguousarray(conn)),
             None, ptr(dof))
    from flexshell import materials
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(E, NU, RHO))
    ctx.call("fs_params_set", _abi.make_params(Dps, Dt, RHO, 0.01, quads=True), None)
    ctx.call("fs_normals_compute")
    nnz = ctypes.c_int64()
    ctx.call("fs_mass", _abi.FS_ASM_DIAG, ctypes.c_int64(nfree), ctypes.byref(nnz))
    m = np.empty(nfree)
    ctx.call("fs_matrix_copy", None, None, ptr(m))
    ctx.call("fs_stiffness", _abi.FS_FP64, _abi.FS_ASM_SPARSE, ctypes.c_int64(nfree), ctypes.byref(nnz))
    om = ctypes.c_double()
    ctx.call("fs_power_iteration", ptr(m), ctypes.c_int64(iters), ctypes.c_uint64(1), ctypes.byref(om))
    dt = 0.9 * 2.0 / om.value
    rng = np.random.Generator(np.random.PCG64(5))
    V0 = np.zeros(nfree)
    wd = dof[:, 2]
    free_w = wd <= nfree
    V0[wd[free_w] - 1] = 1e-3 * np.sin(np.pi * x[free_w]) * np.sin(np.pi * y[free_w]) + rng.normal(0, 1e-5, free_w.sum())
    C = np.zeros(nfree)
    invMC = 1.0 / m
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {}
    finals = {}
    for prec in (_abi.FS_MIXED, _abi.FS_MIXED_COMP, _abi.FS_FP64):
        ctx.call("fs_explicit_setup", prec, ptr(invMC), ptr(C), ctypes.c_double(dt))
        z = np.zeros(nfree)
        ctx.call("fs_explicit_set_state", ptr(z), ptr(V0), ptr(z))
        ctx.call("fs_explicit_run", ctypes.c_int64(64))  # warm-up (graph capture)
        ctx.call("fs_explicit_set_state", ptr(z), ptr(V0), ptr(z))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ctx.call("fs_explicit_run", ctypes.c_int64(nsteps))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        U = np.empty(nfree)
        ctx.call("fs_explicit_get_state", ptr(U), None, None)
        finals[prec] = U
        name = {_abi.FS_MIXED: "mixed", _abi.FS_MIXED_COMP: "mixed_comp", _abi.FS_FP64: "fp64"}[prec]
        out["steps_per_s_" + name] = nsteps / (ms * 1e-3)
        out["ms_per_step_" + name] = ms / nsteps
    U32, U64 = finals[_abi.FS_MIXED], finals[_abi.FS_FP64]
    Uc = finals[_abi.FS_MIXED_COMP]
    # algorithmic bytes of one step on node blocks: the blocks (36 values and a
    # neighbour index each), per node its block range and dofs, per dof the
    # double state read and written by the two kernels and the displacement
    # copy (value size es)
    import scipy.sparse as sps
    nn_ = xyz.shape[0]
    rows_ = np.repeat(np.arange(conn.shape[0]), conn.shape[1])
    inc = sps.csr_matrix((np.ones(rows_.size), (rows_, conn.ravel() - 1)), shape=(conn.shape[0], nn_))
    nblocks = int((inc.T @ inc).nnz)
    bsr_bytes = lambda es: nblocks * (36 * es + 4) + nn_ * (8 + 6 * 4) + nfree * (13 * 8 + 4 + es)
    out.update({"elements": conn.shape[0], "dofs": nfree, "nnz": nnz.value, "steps": nsteps,
                "omega_max": om.value, "dt": dt, "power_iterations": iters,
                "final_u_rel_err_mixed_vs_fp64": float(np.abs(U32 - U64).max() / np.abs(U64).max()),
                "final_u_rel_err_mixed_comp_vs_fp64": float(np.abs(Uc - U64).max() / np.abs(U64).max()),
                "mixed_comp": "float block values with bf16 residuals, float-pair displacement copy, compensated "
                              "float sum of K U",
                "final_u_max": float(np.abs(U64).max()),
                "format": "6x6 node blocks (block rows = node neighbour lists)", "blocks": nblocks,
                "bytes_per_step_mixed": bsr_bytes(4), "bytes_per_step_fp64": bsr_bytes(8),
                "hbm_gbs_mixed": bsr_bytes(4) * out["steps_per_s_mixed"] / 1e9,
                "bytes_per_step_mixed_comp": bsr_bytes(6) + 6 * nn_ * 2,
                "hbm_gbs_mixed_comp": (bsr_bytes(6) + 6 * nn_ * 2) * out["steps_per_s_mixed_comp"] / 1e9,
                "hbm_gbs_fp64": bsr_bytes(8) * out["steps_per_s_fp64"] / 1e9})
    ctx.close()
    return out


def cylinder_panels(npanels=64, seed=3):
    """The reference's configuration 3: cylindrical panels (R 25, L 50, 80 deg
    arc, mapped as test/test_shell_statics.jl:28-33), each an n x n quad grid
    split into 2 n^2 T3FF triangles with n ~ U{16..256}, thickness
    ~ U[0.1, 0.5]; E = 4.32e8, nu = 0."""
    from flexshell import mesh
    rng = np.random.Generator(np.random.PCG64(seed))
    R, L, arc = 25.0, 50.0, 80.0 / 180.0 * np.pi
    panels = []
    for _ in range(npanels):
        n = int(rng.integers(16, 257))
        t = float(rng.uniform(0.1, 0.5))
        xy, conn = mesh.T3block(arc, L, n, n)
        a, y = xy[:, 0], xy[:, 1]
        xyz = np.stack([R * np.sin(a), y, R * (np.cos(a) - 1)], 1)
        panels.append((xyz, conn, t))
    return panels


def batched_c3(torch, device=0, steps=5, warmup=3):
    from flexshell import _abi, materials
    from flexshell._lib import Context, ptr
    panels = cylinder_panels()
    Dps, Dt = materials.shell_material_stiffness(materials.MatDeforElastIso(4.32e8, 0.0))
    prm = _abi.make_params(Dps, Dt, 0.0, 0.0)
    # the batch API (fs_batch_*): one element launch over the work-list of all
    # panels' elements and one gather launch, each panel with its own dofs
    ctx = Context(device)
    ctx.call("fs_params_set", prm, None)
    xyzs = [np.asfortranarray(p[0]) for p in panels]
    conns = [np.ascontiguousarray(p[1]) for p in panels]
    dofs = [np.asfortranarray(np.arange(1, 6 * x.shape[0] + 1, dtype=np.int64).reshape(-1, 6)) for x in xyzs]
    k = len(panels)
    arr = lambda vals, t: (t * k)(*vals)
    vp = ctypes.c_void_p
    ctx.call("fs_batch_set", _abi.FS_T3FF, k, arr([x.shape[0] for x in xyzs], ctypes.c_int64),
             arr([x.ctypes.data for x in xyzs], vp), arr([c.shape[0] for c in conns], ctypes.c_int64),
             arr([c.ctypes.data for c in conns], vp), arr([d.ctypes.data for d in dofs], vp),
             arr([6 * x.shape[0] for x in xyzs], ctypes.c_int64), arr([p[2] for p in panels], ctypes.c_double))
    nel = sum(c.shape[0] for c in conns)
    nnz = ctypes.c_int64()
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {"panels": len(panels), "elements": nel, "n_range": [int(min(p[1].shape[0] for p in panels)),
                                                             int(max(p[1].shape[0] for p in panels))]}
    tiles = (ctypes.c_int32 * 3)()
    for prec, name in ((_abi.FS_MIXED, "mixed"), (_abi.FS_FP64, "fp64")):
        for _ in range(warmup):
            ctx.call("fs_batch_stiffness", prec, 0, None)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            ctx.call("fs_batch_stiffness", prec, 0, None)
        e1.record(stream)
        torch.cuda.synchronize()
        out["batched_elements_per_s_" + name] = nel / (e0.elapsed_time(e1) / steps * 1e-3)
        ctx.call("fs_tuning", tiles)
        out["tiles_" + name] = {"elements_per_block": tiles[0], "gather_warps": tiles[1], "tuned": bool(tiles[2])}
    ctx.close()
    # one context and one call per panel
    ctxs = []
    for xyz_p, conn_p, t in panels:
        c = Context(device)
        xp = np.asfortranarray(xyz_p)
        dp = np.asfortranarray(np.arange(1, 6 * xp.shape[0] + 1, dtype=np.int64).reshape(-1, 6))
        c.call("fs_mesh_set", _abi.FS_T3FF, xp.shape[0], ptr(xp), conn_p.shape[0], ptr(np.ascontiguousarray(conn_p)),
               None, ptr(dp))
        p2 = _abi.make_params(Dps, Dt, 0.0, t)
        c.call("fs_params_set", p2, None)
        c.call("fs_normals_compute")
        ctxs.append((c, 6 * xp.shape[0]))
    for prec, name in ((_abi.FS_MIXED, "mixed"), (_abi.FS_FP64, "fp64")):
        for c, nn in ctxs:
            c.call("fs_stiffness", prec, 0, ctypes.c_int64(nn), ctypes.byref(nnz))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            for c, nn in ctxs:
                c.call("fs_stiffness", prec, 0, ctypes.c_int64(nn), ctypes.byref(nnz))
        torch.cuda.synchronize()
        out["per_mesh_elements_per_s_" + name] = nel / ((time.perf_counter() - t0) / steps)
    for c, _ in ctxs:
        c.close()
    return out


def corotbeam_lattice(torch, device=0, n=100, steps=5, warmup=3):
    """FEMMCorotBeam throughput: beams along the edges of an n^3 lattice
    (3 n^2 (n-1) elements) in a deformed state (random displacements and
    nodal rotations), double precision; device time of the element kernel +
    CSR gather for each matrix, and of the restoring-force kernels."""
    from flexshell import _abi
    from flexshell._lib import Context, ptr
    rng = np.random.Generator(np.random.PCG64(7))
    g = np.arange(n, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.asfortranarray(np.column_stack([X.ravel(), Y.ravel(), Z.ravel()]) + rng.uniform(-0.1, 0.1, (n ** 3, 3)))
    idx = np.arange(1, n ** 3 + 1).reshape(n, n, n)
    conn = np.ascontiguousarray(np.concatenate(
        [np.column_stack([np.moveaxis(idx, a, 0)[:-1].ravel(), np.moveaxis(idx, a, 0)[1:].ravel()])
         for a in range(3)]), dtype=np.int64)
    ne, nn = conn.shape[0], xyz.shape[0]
    sec = (_abi.fs_beam_section * ne)()
    arr = np.frombuffer(sec, dtype=np.float64).reshape(ne, 10)
    arr[:, 0], arr[:, 2], arr[:, 3] = 0.01, 1e-5, 2e-5
    arr[:, 1] = arr[:, 2] + arr[:, 3]
    arr[:, 4], arr[:, 5], arr[:, 6] = 2.5e-5, np.inf, np.inf
    arr[:, 7:] = rng.normal(size=(ne, 3))
    dof = np.asfortranarray(np.arange(1, 6 * nn + 1, dtype=np.int64).reshape(nn, 6))
    u1 = np.asfortranarray(rng.uniform(-0.01, 0.01, (nn, 3)))
    # nodal rotations (Rodrigues) of small random rotation vectors, R[:] per node
    a = rng.normal(scale=0.05, size=(nn, 3))
    th = np.linalg.norm(a, axis=1)[:, None, None]
    S = np.zeros((nn, 3, 3))
    S[:, 0, 1], S[:, 0, 2], S[:, 1, 2] = -a[:, 2], a[:, 1], -a[:, 0]
    S = S - S.transpose(0, 2, 1)
    R = np.eye(3) + np.sin(th) / th * S + (1 - np.cos(th)) / th ** 2 * (S @ S)
    R1 = np.asfortranarray(R.transpose(0, 2, 1).reshape(nn, 9))
    v1 = np.asfortranarray(rng.normal(size=(nn, 6)))
    ctx = Context(device)
    ctx.call("fs_mesh_set", _abi.FS_COROTBEAM, nn, ptr(xyz), ne, ptr(conn), None, ptr(dof))
    ctx.call("fs_beam_setup", sec, 2.1e11, 0.3, 7850.0)
    ctx.call("fs_beam_state_set", ptr(u1), ptr(R1), ptr(v1))
    nnz = ctypes.c_int64()
    t = np.zeros(4)
    out = {"elements": ne, "nodes": nn, "lattice": n}
    for which, name in ((_abi.FS_BEAM_STIFFNESS, "stiffness"), (_abi.FS_BEAM_GEOSTIFFNESS, "geostiffness"),
                        (_abi.FS_BEAM_MASS, "mass"), (_abi.FS_BEAM_GYROSCOPIC, "gyroscopic")):
        for _ in range(warmup):
            ctx.call("fs_beam_matrix", which, 1, 0, 6 * nn, ctypes.byref(nnz))
        el = ga = 0.0
        for _ in range(steps):
            ctx.call("fs_beam_matrix", which, 1, 0, 6 * nn, ctypes.byref(nnz))
            ctx.call("fs_timings", ptr(t), 4)
            el += t[0]
            ga += t[1]
        out[name] = {"elements_per_s": ne / ((el + ga) / steps * 1e-3), "ms_elements": el / steps,
                     "ms_gather": ga / steps}
    out["nnz"] = nnz.value
    F = np.empty(6 * nn)
    for _ in range(warmup):
        ctx.call("fs_beam_restoringforce", 6 * nn, ptr(F))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.call("fs_beam_restoringforce", 6 * nn, ptr(F))
    out["restoringforce_elements_per_s_incl_d2h"] = ne / ((time.perf_counter() - t0) / steps)
    ctx.close()
    return out


def composite_c4(torch, device=0, n=512, n_eig=512, nev=20, steps=5, warmup=3, n_eig_t3=256):
    """The layered Q4RS plate ([0/90/90/0], 0.25 mm plies, 1 m side, simply
    supported, in-plane rigid-body motion restrained): stiffness assembly in
    the three arithmetic modes at n x n, and the nev lowest eigenvalues of an
    n_eig x n_eig plate from the FP64, compensated mixed and plain mixed
    stiffness with the lumped mass: ARPACK shift-invert (SciPy's eigsh, the
    library behind the reference's eigs) about -1, with K - sigma M
    factorised and solved on the GPU (flexshell.eigs); and the same 20
    eigenvalues of an n_eig_t3 x n_eig_t3 plate with its quads split in
    triangles (T3FFComp), FP64 and compensated."""
    from flexshell import _abi, materials, mesh
    from flexshell.eigen import eigs
    from flexshell.femm import (FEMMShellQ4RSComp, FEMMShellT3FFComp, NodalField, SysmatAssemblerSparse,
                                SysmatAssemblerSparseSymm)
    from flexshell._lib import laminate, ptr
    lam = materials.lamina_material(1600.0, 140e9, 10e9, 0.3, 5e9, 5e9, 3.5e9)
    Dps, Dts = materials.shell_material_stiffness(lam)
    g = laminate([dict(Dps=Dps, Dts=Dts, thickness=0.25e-3, angle=a, rho=1600.0) for a in (0, 90, 90, 0)])

    def plate_c4(m, triangles=False):
        xy, conn = mesh.Q4block(1.0, 1.0, m, m)
        xyz = mesh.xyz3(xy)
        x, y = xyz[:, 0], xyz[:, 1]
        tol = 1.0 / m / 100
        bnd = (np.abs(x) < tol) | (np.abs(x - 1) < tol) | (np.abs(y) < tol) | (np.abs(y - 1) < tol)
        fixed = np.zeros((xyz.shape[0], 6), bool)
        fixed[bnd, 2] = True
        # in-plane rigid-body motion restrained: u = v = 0 at (0, 0), v = 0 at (1, 0)
        c0, c1 = int(np.argmin(np.abs(x) + np.abs(y))), int(np.argmin(np.abs(x - 1) + np.abs(y)))
        fixed[c0, 0] = fixed[c0, 1] = fixed[c1, 1] = True
        dof, nfree = mesh.numberdofs(fixed)
        femm = (FEMMShellT3FFComp(mesh.quads_to_triangles(conn), g, device=device) if triangles
                else FEMMShellQ4RSComp(conn, g, device=device))
        geom0 = NodalField(xyz)
        dchi = NodalField(np.zeros((xyz.shape[0], 6)))
        dchi.dofnums = np.asfortranarray(dof)
        femm.associategeometry(geom0)
        return femm, geom0, dchi, nfree

    out = {"elements": n * n, "eig_elements": n_eig * n_eig, "nev": nev}
    femm, geom0, dchi, nfree = plate_c4(n)
    asm = SysmatAssemblerSparse()
    t = np.zeros(4)
    for prec, name in ((_abi.FS_MIXED, "mixed"), (_abi.FS_MIXED_COMP, "mixed_comp"), (_abi.FS_FP64, "fp64")):
        for _ in range(warmup):
            femm.stiffness(asm, geom0, None, None, dchi, precision=prec)
        ms = 0.0
        for _ in range(steps):
            nnz = ctypes.c_int64()
            femm.ctx.call("fs_stiffness", prec, 0, dchi.nalldofs(), ctypes.byref(nnz))
            femm.ctx.call("fs_timings", ptr(t), 4)
            ms += t[0] + t[1]
        out["stiffness_elements_per_s_" + name] = n * n / (ms / steps * 1e-3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    femm.mass(SysmatAssemblerSparseSymm(), geom0, dchi)
    out["mass_ms_incl_copy"] = 1e3 * (time.perf_counter() - t0)
    femm.close()
    femm, geom0, dchi, nfree = plate_c4(n_eig)
    out["eig_dofs"] = nfree
    from flexshell._lib import FlexShellError
    w = {}
    for prec, name in ((_abi.FS_FP64, "fp64"), (_abi.FS_MIXED_COMP, "mixed_comp"), (_abi.FS_MIXED, "mixed")):
        t0 = time.perf_counter()
        try:
            w[name] = eigs(femm, geom0, dchi, nev, sigma=-1.0, precision=prec, nfree=nfree, tol=1e-12,
                           return_eigenvectors=False)
        except FlexShellError as e:
            # the stiffness of this mode has eigenvalues below the shift (its
            # rounding is not of the Gram form and lifts or lowers the soft modes)
            out["eig_error_" + name] = str(e)
        out["eig_seconds_" + name] = time.perf_counter() - t0
    femm.close()
    for name in ("mixed_comp", "mixed"):
        out["eig_rel_err_%s_vs_fp64_max" % name] = (
            float((np.abs(w[name] - w["fp64"]) / np.abs(w["fp64"])).max()) if name in w else None)
    out["M_rel_err_mixed_vs_fp64_max"] = 0.0  # the lumped mass is double in every mode
    out["lowest_hz"] = float(np.sqrt(w["fp64"][0]) / (2 * np.pi))
    # the same plate with its quads split in triangles (T3FFComp: the element
    # type of the headline step, whose compensated sums are Dot2): the 20
    # lowest eigenvalues in FP64 and the compensated mode
    femm, geom0, dchi, nfree = plate_c4(n_eig_t3, triangles=True)
    wt = {}
    for prec, name in ((_abi.FS_FP64, "fp64"), (_abi.FS_MIXED_COMP, "mixed_comp")):
        wt[name] = eigs(femm, geom0, dchi, nev, sigma=-1.0, precision=prec, nfree=nfree, tol=1e-12,
                        return_eigenvectors=False)
    femm.close()
    out["t3_eig_elements"] = 2 * n_eig_t3 * n_eig_t3
    out["t3_eig_rel_err_mixed_comp_vs_fp64_max"] = float(
        (np.abs(wt["mixed_comp"] - wt["fp64"]) / np.abs(wt["fp64"])).max())
    out["eigensolver"] = ("ARPACK shift-invert (scipy eigsh) about -1, K - sigma M factorised on the GPU "
                          "(banded Cholesky, double)")
    out["boundary"] = "w = 0 on the edges; u = v = 0 at (0,0), v = 0 at (1,0)"
    return out


def time_steps(asm, precision, steps, warmup, torch, stream):
    for _ in range(warmup):
        asm.stiffness(precision)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phases = np.zeros(4)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        nnz = asm.stiffness(precision)
        phases += asm.timings()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / steps, phases / steps, nnz


def t3_bytes(nelem, nnz, nodes, precision, pairs_once):
    """Algorithmic bytes of one launch of each kernel of the T3FF step.

    Element kernel: connectivity (3 x 4), coordinates (3 x 24), double normals
    (3 x 24; the mixed modes also their float copy, 3 x 12), validity flags
    (3) and thickness (8) in; the 6 upper 6x6 node blocks out (4 bytes an
    entry for FS_MIXED, 8 for a float pair or a double).  Gather: the node
    blocks it sums (each of the 6 upper blocks once when the node-block pairs
    are summed once, else the 9 blocks, mirrored ones included), the double
    CSR values out, the pair lists and slots (3 x 8 per element), per node its
    dofs, offsets, row length and row pointers, and the column map (2 bytes a
    row position)."""
    from flexshell import _abi
    es = 4 if precision == _abi.FS_MIXED else 8
    el_in = 3 * 4 + 3 * 24 + 3 * 24 + 3 + 8 + (3 * 12 if precision != _abi.FS_FP64 else 0)
    elem = nelem * (el_in + 216 * es)
    blocks = 216 if pairs_once else 324
    gather = (nelem * blocks * es + nnz * 8 + nelem * 3 * 8 + nodes * (6 * 4 + 8 + 4 + 8 + 6 * 8)
              + 2 * nnz // 6)
    return elem, gather


def survey_step_bytes(nelem, nnz):
    """The minimal bytes of one T3FF stiffness assembly (the per-element
    work model of the hot path): inputs connectivity 3 x 4, coordinates 72,
    normals 72, flags 3 per element, and the double CSR values out."""
    return nelem * (3 * 4 + 72 + 72 + 3) + nnz * 8


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--n", type=int, default=1024, help="quads per side")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-oracle", action="store_true", help="skip the full-size FP64 check against the oracle")
    ap.add_argument("--no-explicit", action="store_true")
    ap.add_argument("--eig-n", type=int, default=512,
                    help="quads per side of the layered plate of the 20-eigenvalue check (512, the default: the "
                         "reference's configuration, 1.58 M dofs, a 45 GB band factor per mode, about three "
                         "minutes for the three modes)")
    ap.add_argument("--explicit-only", action="store_true",
                    help="only the explicit-dynamics section, on an n x n Q4RS plate for 64 x steps steps "
                         "(a small case for profiling the step kernels)")
    ap.add_argument("--assembly-only", choices=["mixed", "mixed_comp", "fp64"],
                    help="only warmup + steps stiffness assemblies of the n x n plate in one arithmetic mode "
                         "(a small case for profiling the element and gather kernels)")
    ap.add_argument("--quads", action="store_true", help="with --assembly-only: Q4RS instead of T3FF")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.explicit_only:
        import torch
        print(json.dumps(explicit_c5(torch, device=0, n=args.n, nsteps=64 * args.steps, iters=50)))
        return 0
    if args.assembly_only:
        import torch
        from flexshell import _abi
        prec = {"mixed": _abi.FS_MIXED, "mixed_comp": _abi.FS_MIXED_COMP, "fp64": _abi.FS_FP64}[args.assembly_only]
        xyz, conn, dof = plate(args.n, args.quads)
        a = Assembler(xyz, conn, dof, args.quads)
        ms, ph, nnz = time_steps(a, prec, args.steps, args.warmup, torch,
                                 torch.cuda.ExternalStream(a.ctx.stream()))
        print(json.dumps({"mode": args.assembly_only, "quads": args.quads, "n": args.n, "elements": conn.shape[0],
                          "nnz": nnz, "ms_per_step": ms, "ms_elements": ph[0], "ms_gather": ph[1],
                          "tiles": a.tiles()}))
        a.ctx.close()
        return 0

    import torch
    import torch.distributed as dist
    from flexshell import _abi
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    HEAD = _abi.FS_MIXED_COMP  # the mode behind `value`

    res = {}
    # --- T3FF (headline) -----------------------------------------------------
    xyz, conn, dof = plate(args.n, False)
    asm = Assembler(xyz, conn, dof, False, device=local)
    stream = torch.cuda.ExternalStream(asm.ctx.stream())
    nnz0 = asm.stiffness(HEAD)  # builds the pattern
    t_sym = asm.timings()[2]
    # page-locked host arrays of the end-to-end leg, allocated before the large
    # host copies of the precision checks below: freshly allocated, while the
    # host is still returning those pages, they copied 20 % slower
    nn = xyz.shape[0]
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    h_xyz = pin((3 * nn,), torch.float64)
    h_xyz[:] = xyz.flatten(order="F")
    h_dof = pin((6 * nn,), torch.int64)
    h_dof[:] = dof.flatten(order="F")
    h_colptr = pin((asm.n + 1,), torch.int64)
    h_rowval = pin((nnz0,), torch.int64)
    h_nzval = pin((nnz0,), torch.float64)
    # the host's device-to-host copy rate at this moment (a 1 GiB copy into
    # page-locked memory, best of three): the end-to-end step is bound by its
    # 4.3 GB copy back, and the host's memory is shared with other jobs
    d_probe = torch.ones(1 << 27, dtype=torch.float64, device="cuda")
    h_probe = torch.empty(1 << 27, dtype=torch.float64, pin_memory=True)
    d2h_gbs = 0.0
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h_probe.copy_(d_probe, non_blocking=True)
        torch.cuda.synchronize()
        d2h_gbs = max(d2h_gbs, (1 << 30) / (time.perf_counter() - t0) / 1e9)
    del d_probe, h_probe
    if world > 1:
        dist.barrier()
    # clocks sampled over every timed region of the T3FF section (the headline
    # step, the other modes' steps and the end-to-end steps)
    clocks = Clocks(local)
    clocks.__enter__()
    # --- e2e through the C ABI from pinned host buffers (T3FF, headline mode),
    # timed before the precision checks' multi-GB host copies below ---
    P = asm.ptr

    def e2e_step():
        asm.ctx.call("fs_geometry_set", P(h_xyz))
        asm.ctx.call("fs_dofs_set", P(h_dof))
        k = ctypes.c_int64()
        asm.ctx.call("fs_pattern", asm.n, ctypes.byref(k))
        asm.ctx.call("fs_stiffness_copy", HEAD, asm.n, P(h_colptr), P(h_rowval), P(h_nzval))

    # more warm-up than the device-timed steps: the first copies into freshly
    # pinned host pages ran up to 20 % slower
    for _ in range(max(args.warmup, 6)):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    ms_e2e = 1e3 * (time.perf_counter() - t0) / args.steps
    ms_e2e = max_over_ranks(ms_e2e, world, dist)
    h2d = (3 * nn) * 8 + (6 * nn) * 8
    d2h = (asm.n + 1) * 8 + nnz0 * 8 + nnz0 * 8
    del h_colptr, h_rowval, h_nzval
    ms_head, ph_head, nnz = time_steps(asm, HEAD, args.steps, args.warmup, torch, stream)
    ms_head = max_over_ranks(ms_head, world, dist)
    tiles_head = asm.tiles()
    v_head = asm.values(nnz)
    ms_fp64, ph_fp64, _ = time_steps(asm, _abi.FS_FP64, args.steps, args.warmup, torch, stream)
    tiles_fp64 = asm.tiles()
    v_fp64 = asm.values(nnz)
    err_head = float(np.abs(v_head - v_fp64).max() / np.abs(v_fp64).max())
    fro_head = float(np.linalg.norm(v_head - v_fp64) / np.linalg.norm(v_fp64))
    del v_head
    ms_mx, ph_mx, _ = time_steps(asm, _abi.FS_MIXED, args.steps, args.warmup, torch, stream)
    tiles_mx = asm.tiles()
    v_mx = asm.values(nnz)
    err_mx = float(np.abs(v_mx - v_fp64).max() / np.abs(v_fp64).max())
    del v_mx, v_fp64
    clocks.__exit__(None, None, None)

    oracle_t3 = None
    if not args.no_oracle and rank == 0:
        oracle_t3 = oracle_check_c2(asm, xyz, conn, dof, False, nnz)
    res["t3"] = dict(ms_head=ms_head, ms_fp64=ms_fp64, ph_head=ph_head, ph_fp64=ph_fp64, nnz=nnz,
                     err=err_head, fro=fro_head, t_sym=t_sym, nelem=conn.shape[0],
                     ms_mx=ms_mx, ph_mx=ph_mx, err_mx=err_mx,
                     tiles={"mixed_comp": tiles_head, "fp64": tiles_fp64, "mixed": tiles_mx})
    asm.ctx.close()
    del asm

    # --- Q4RS -------------------------------------------------------------------
    xyz, conn, dof = plate(args.n, True)
    asm = Assembler(xyz, conn, dof, True, device=local)
    stream = torch.cuda.ExternalStream(asm.ctx.stream())
    asm.stiffness(HEAD)
    t_sym_q4 = asm.timings()[2]
    ms_q_head, ph_q_head, nnz_q = time_steps(asm, HEAD, args.steps, args.warmup, torch, stream)
    tiles_q = {"mixed_comp": asm.tiles()}
    vq_h = asm.values(nnz_q)
    ms_q_fp64, ph_q_fp64, _ = time_steps(asm, _abi.FS_FP64, args.steps, args.warmup, torch, stream)
    tiles_q["fp64"] = asm.tiles()
    vq_d = asm.values(nnz_q)
    err_q4 = float(np.abs(vq_h - vq_d).max() / np.abs(vq_d).max())
    del vq_h
    ms_q_mx, ph_q_mx, _ = time_steps(asm, _abi.FS_MIXED, args.steps, args.warmup, torch, stream)
    tiles_q["mixed"] = asm.tiles()
    vq_m = asm.values(nnz_q)
    err_q4m = float(np.abs(vq_m - vq_d).max() / np.abs(vq_d).max())
    del vq_m, vq_d
    oracle_q4 = None
    if not args.no_oracle and rank == 0:
        oracle_q4 = oracle_check_c2(asm, xyz, conn, dof, True, nnz_q)
    asm.ctx.close()
    del asm

    ex = explicit_c5(torch, device=local) if not args.no_explicit else None
    bc3 = batched_c3(torch, device=local) if not args.no_explicit else None
    beams = corotbeam_lattice(torch, device=local) if not args.no_explicit else None
    c4 = composite_c4(torch, device=local, n_eig=args.eig_n) if not args.no_explicit else None
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0
    t3 = res["t3"]
    ne3, ne4 = t3["nelem"], conn.shape[0]
    value = world * ne3 / (ms_head * 1e-3)
    # roofline of the dominant kernel of the headline step
    hbm, peak_kind = read_peaks()
    el_ms, ga_ms = t3["ph_head"][0], t3["ph_head"][1]
    nodes = (args.n + 1) ** 2
    pairs_once = t3["tiles"]["mixed_comp"]["pairs_once"]
    el_bytes, ga_bytes = t3_bytes(ne3, nnz, nodes, HEAD, pairs_once)
    step_bytes = survey_step_bytes(ne3, nnz)
    mode = {_abi.FS_MIXED: "FS_MIXED", _abi.FS_MIXED_COMP: "FS_MIXED_COMP", _abi.FS_FP64: "FS_FP64"}[HEAD]
    if el_ms >= ga_ms:
        dom, ms_dom, own = "k_t3_elements " + mode, el_ms, el_bytes
    else:
        dom, ms_dom, own = "k_gather " + mode, ga_ms, ga_bytes
    achieved = step_bytes / (ms_dom * 1e-3) / 1e9
    traffic, traffic_src = measured_traffic(dom, ne3)
    tr_el, _ = measured_traffic("k_t3_elements " + mode, ne3)
    tr_ga, _ = measured_traffic("k_gather " + mode, ne3)
    cb = cb1 = None
    if not args.no_cpu:
        cb, _ = cpu_baseline(steps=1, n=args.n)
        cb1, _ = cpu_baseline(steps=1, n=args.n, nthreads=1)
        cb["single_thread_value"] = cb1["value"]
        cb["single_thread_sample"] = cb1["sample"]
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_head, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-element (compensated, float pairs)/f64-assembly", "data": "synthetic",
        "config": {"workload": workload_text(args.n),
                   "elements": ne3, "nnz": nnz, "precision": "FS_MIXED_COMP", "assembler": "SysmatAssemblerSparse",
                   "pattern": "built once per mesh (symbolic %.2f ms), not in the timed step" % t3["t_sym"],
                   "l2": "inputs larger than L2 (element matrices %.2f GB, values %.2f GB)" % (
                       ne3 * 216 * 8 / 1e9, nnz * 8 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": world * ne3 / (ms_e2e * 1e-3), "unit": "elements/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e,
                "host_d2h_gbs": d2h_gbs, "ms_copy_back_at_host_rate": d2h / (d2h_gbs * 1e9) * 1e3,
                "path": "C ABI from pinned host: fs_geometry_set + fs_dofs_set + fs_pattern (pattern "
                        "rebuilt) + fs_stiffness_copy (FS_MIXED_COMP; CSC copied back, pattern copy "
                        "overlapping the kernels)"},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "algorithmic_bytes_per_launch": step_bytes,
                     "algorithmic_bytes_basis": "minimal bytes of the whole assembly per element (inputs 159 B "
                                                "+ 8 B per stored value) x elements, over the dominant "
                                                "kernel's time",
                     "ms_per_launch": ms_dom,
                     "frac_step": step_bytes / (ms_head * 1e-3) / 1e9 / hbm,
                     "frac_kernel_own_bytes": own / (ms_dom * 1e-3) / 1e9 / hbm,
                     "kernel_own_bytes_per_launch": own,
                     "traffic_step_over_algorithmic": ((tr_el + tr_ga) / step_bytes
                                                       if tr_el is not None and tr_ga is not None else None)},
        "clocks": dict(clocks.summary(), window="the T3FF timed regions: the three modes' steps, e2e steps"),
        "cpu_baseline": cb,
        "accuracy_of_value_mode": {
            "mode": "FS_MIXED_COMP",
            "K_rel_err_vs_fp64_max": t3["err"],
            "M_rel_err_vs_fp64_max": 0.0,
            "eig20_rel_err_vs_fp64_max": c4["eig_rel_err_mixed_comp_vs_fp64_max"] if c4 else None,
            "eig20_plate": ("layered Q4RS plate, %d x %d quads" % ((int(round(np.sqrt(c4["eig_elements"]))),) * 2))
                           if c4 else None,
            "eig20_t3_rel_err_vs_fp64_max": c4["t3_eig_rel_err_mixed_comp_vs_fp64_max"] if c4 else None,
            "eig20_t3_plate": ("the same plate as T3FFComp, %d triangles" % c4["t3_eig_elements"]) if c4 else None},
        "results": {
            "t3ff": {"elements": ne3, "nnz": nnz,
                     "mixed_comp_elements_per_s": ne3 / (ms_head * 1e-3),
                     "mixed_comp_over_fp64": ms_fp64 / ms_head,
                     "nnz_per_s_mixed_comp": nnz / (ms_head * 1e-3),
                     "rel_err_K_mixed_comp_vs_fp64_max": t3["err"], "rel_err_K_mixed_comp_vs_fp64_fro": t3["fro"],
                     "ms_elements_mixed_comp": t3["ph_head"][0], "ms_gather_mixed_comp": t3["ph_head"][1],
                     "fp64_elements_per_s": ne3 / (ms_fp64 * 1e-3),
                     "ms_elements_fp64": t3["ph_fp64"][0], "ms_gather_fp64": t3["ph_fp64"][1],
                     "mixed_elements_per_s": ne3 / (t3["ms_mx"] * 1e-3),
                     "mixed_over_fp64": ms_fp64 / t3["ms_mx"],
                     "rel_err_K_mixed_vs_fp64_max": t3["err_mx"],
                     "ms_elements_mixed": t3["ph_mx"][0], "ms_gather_mixed": t3["ph_mx"][1],
                     "rel_err_M_mixed_vs_fp64_max": 0.0,
                     "ms_symbolic": t3["t_sym"], "e2e_ms": ms_e2e, "tiles": t3["tiles"],
                     "fp64_vs_oracle": oracle_t3},
            "q4rs": {"elements": ne4, "nnz": nnz_q,
                     "mixed_comp_elements_per_s": ne4 / (ms_q_head * 1e-3),
                     "mixed_comp_over_fp64": ms_q_fp64 / ms_q_head,
                     "rel_err_K_mixed_comp_vs_fp64_max": err_q4,
                     "ms_elements_mixed_comp": ph_q_head[0], "ms_gather_mixed_comp": ph_q_head[1],
                     "fp64_elements_per_s": ne4 / (ms_q_fp64 * 1e-3),
                     "ms_elements_fp64": ph_q_fp64[0], "ms_gather_fp64": ph_q_fp64[1],
                     "mixed_elements_per_s": ne4 / (ms_q_mx * 1e-3), "mixed_over_fp64": ms_q_fp64 / ms_q_mx,
                     "rel_err_K_mixed_vs_fp64_max": err_q4m,
                     "ms_elements_mixed": ph_q_mx[0], "ms_gather_mixed": ph_q_mx[1],
                     "ms_symbolic": t_sym_q4, "tiles": tiles_q, "fp64_vs_oracle": oracle_q4},
            "explicit_q4rs_512": ex,
            "batched_64_cylinder_panels": bc3,
            "corotbeam_lattice_100": beams,
            "composite_q4rs_512": c4,
        },
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

// Numeric phase: element-matrix dispatch, nodal normals, lumped mass and
// the tile-shape autotuner.  The kernels of the element matrices are in
// fs_elem_t3.cu and fs_elem_q4.cu, the CSR gather in fs_gather.cu.
//
// Element matrices.  One thread owns one T3 element (or one quadrature point
// of a Q4 element, four lanes per element).  It writes the element's Gram
// rows (csrc/fs_elem_math.cuh) into its own slice of shared memory and then
// forms K = Bh^T Bh as 6x6 node blocks.  The matrix is symmetric, so only its
// upper node blocks (a <= b) are stored, by assembly rank, row-major inside a
// block (6 of 9 blocks for T3, 10 of 16 for Q4); the gather reads a lower
// block as the transpose of its mirror.
//
// Gather.  One warp owns one node, i.e. the six CSR rows of its dofs.  It
// walks the node's (element, local node) pairs in ascending assembly rank
// and adds each slab into a double accumulator, so every CSR value is the
// left-to-right sum of its element contributions in assembly order, as
// Julia's sparse(I, J, V) combines duplicates.  No atomics: the result is
// bitwise reproducible.
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "fs_elem_common.cuh"

namespace fs {

// Shared memory of one block of the element kernels (per-element Gram rows).
size_t t3_smem(int precision, bool avgk, bool layered, int epb)
{
    const int nr = avgk ? T3Rows<true>::N : T3Rows<false>::N;
    const int per = layered ? nr * 18 + 1
                            : (avgk ? CompactRows<3, T3Rows<true>::NS>::SIZE : CompactRows<3, T3Rows<false>::NS>::SIZE) + 1;
    return (precision == FS_FP64 ? 8 : 4) * (size_t)epb * per;
}

// element kernels of one precision into `ke` (the layout of the element buffer)
static int run_elements(fs_ctx *c, int precision, void *ke)
{
    return c->mesh.nen == 3 ? run_t3_any(c, precision, ke) : run_q4_any(c, precision, ke);
}

// bytes of one stored element-matrix entry
size_t entry_bytes(int precision) { return precision == FS_MIXED ? 4 : 8; }

int launch_elements(fs_ctx *c, int precision)
{
    MeshDev &m = c->mesh;
    size_t bytes = (size_t)m.nelem * n_upper_blocks(m.nen) * 36 * entry_bytes(precision);
    if (bytes > c->ke_bytes) {
        if (c->ke) cudaFree(c->ke);
        c->ke = nullptr;
        c->ke_bytes = 0;
        cudaError_t e = cudaMalloc(&c->ke, bytes ? bytes : 16);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_err(c, FS_ERR_OOM, "device allocation of element matrices failed");
        }
        c->ke_bytes = bytes;
    }
    if (m.nelem == 0) return FS_OK;
    return run_elements(c, precision, c->ke);
}

// ---------------------------------------------------------------------------
// nodal normals (associategeometry!)
// ---------------------------------------------------------------------------
// A built-in material csys (the mcsys of associategeometry!): its kind and
// parameters (the FS_CSYS_* values of fs_normals_compute_csys).
struct CsysSpec {
    int kind;
    double prm[9];
};

// third axis of the csys at the point XYZ (cartesian: fixed; cylindrical:
// radial from the axis through prm[0..2] along the unit prm[3..5];
// spherical: radial from the centre prm[0..2])
__device__ void csys_normal(const CsysSpec &cs, const double XYZ[3], double nn[3])
{
    if (cs.kind == FS_CSYS_CARTESIAN) {
        for (int c = 0; c < 3; c++) nn[c] = cs.prm[6 + c];
        return;
    }
    double r[3];
    for (int c = 0; c < 3; c++) r[c] = XYZ[c] - cs.prm[c];
    if (cs.kind == FS_CSYS_CYLINDRICAL) {
        const double d = r[0] * cs.prm[3] + r[1] * cs.prm[4] + r[2] * cs.prm[5];
        for (int c = 0; c < 3; c++) r[c] -= d * cs.prm[3 + c];
    }
    const double l = sqrt(dot3(r, r));
    for (int c = 0; c < 3; c++) nn[c] = r[c] / l;
}

// normal of element `rank` at its node a (times the surface Jacobian for Q4):
// the layup csys axis (layered), the csys normal at the node (a built-in
// mcsys), or the element frame normal (isoparametric)
template <int NN>
__device__ void elem_node_normal(const MeshDev &m, int64_t rank, int a, bool comp, const CsysSpec &cs, double nn[3])
{
    double X[NN][3];
    for (int q = 0; q < NN; q++) {
        int node = m.conn[rank * NN + q];
        for (int c = 0; c < 3; c++) X[q][c] = m.xyz[(int64_t)c * m.nnodes + node];
    }
    double J0[3], J1[3], jac = 1.0;
    if (NN == 3) {
        for (int c = 0; c < 3; c++) {
            J0[c] = X[1][c] - X[0][c];
            J1[c] = X[2][c] - X[0][c];
        }
    } else {
        const double xs[4] = {-1, 1, 1, -1}, ys[4] = {-1, -1, 1, 1};
        double gp[4][2];
        q4_dbasis(xs[a], ys[a], gp);
        for (int c = 0; c < 3; c++) {
            J0[c] = 0;
            J1[c] = 0;
            for (int q = 0; q < NN; q++) {
                J0[c] += X[q][c] * gp[q][0];
                J1[c] += X[q][c] * gp[q][1];
            }
        }
        double cr[3];
        cross3(J0, J1, cr);
        jac = sqrt(dot3(cr, cr));
    }
    if (comp) {
        const double *lc = m.groups[m.group[rank]].csmat;
        for (int c = 0; c < 3; c++) nn[c] = jac * lc[6 + c];
    } else if (cs.kind != FS_CSYS_ISOPARAMETRIC) {
        double v[3];
        csys_normal(cs, X[a], v);
        for (int c = 0; c < 3; c++) nn[c] = jac * v[c];
    } else {
        double e[3][3];
        make_frame(J0, J1, e);
        for (int c = 0; c < 3; c++) nn[c] = jac * e[2][c];
    }
}

// Node sums in assembly order, then the validity test: against the element
// frame normal for T3 (src/FEMMShellT3FFModule.jl:598-611), against the
// mcsys normal at the node for Q4 (src/FEMMShellQ4RSModule.jl:505-519).
template <int NN>
__global__ void k_normals(const MeshDev m, bool comp, double cos_thr, const CsysSpec cs, double *normals,
                          uint8_t *valid)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nnodes) return;
    const CsysSpec iso{FS_CSYS_ISOPARAMETRIC, {0, 0, 0, 0, 0, 0, 0, 0, 0}};
    double s[3] = {0, 0, 0};
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        int32_t v = m.pair_e[p];
        double nn[3];
        elem_node_normal<NN>(m, v >> 2, v & 3, comp, cs, nn);
        for (int c = 0; c < 3; c++) s[c] += nn[c];
    }
    double len = sqrt(dot3(s, s));
    if (len > 0.0)
        for (int c = 0; c < 3; c++) s[c] /= len;
    bool ok = true;
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        int32_t v = m.pair_e[p];
        double nn[3];
        elem_node_normal<NN>(m, v >> 2, v & 3, comp, NN == 3 ? iso : cs, nn);
        if (NN == 4) {  // the validity test uses the unit normal at the node
            double l = sqrt(dot3(nn, nn));
            if (l > 0.0)
                for (int c = 0; c < 3; c++) nn[c] /= l;
        }
        if (dot3(s, nn) < cos_thr) ok = false;
    }
    for (int c = 0; c < 3; c++) normals[(int64_t)c * m.nnodes + r] = s[c];
    valid[r] = ok ? 1 : 0;
}

__global__ void k_round_normals(int64_t n, const double *src, float *dst)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

// the float copy of the normals read by the float rows' triads
int round_normals(fs_ctx *c)
{
    const MeshDev &m = c->mesh;
    if (m.nnodes == 0) return FS_OK;
    k_round_normals<<<nblk2(3 * m.nnodes, 256), 256, 0, c->stream>>>(3 * m.nnodes, m.normals, m.normals_f);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

int launch_normals(fs_ctx *c, int kind, const double *prm)
{
    MeshDev &m = c->mesh;
    CsysSpec cs{kind, {0, 0, 0, 0, 0, 0, 0, 0, 0}};
    const int np = kind == FS_CSYS_CARTESIAN ? 9 : (kind == FS_CSYS_CYLINDRICAL ? 6 : (kind == FS_CSYS_SPHERICAL ? 3 : 0));
    for (int k = 0; k < np; k++) cs.prm[k] = prm[k];
    if (m.nnodes == 0) return FS_OK;
    double th = c->params.threshold_angle;
    double sn = sin(th / 180.0 * M_PI);
    double ntol = 1 - sqrt(1 - sn * sn);
    double cos_thr = 1 - ntol;
    bool comp = (m.etype == FS_T3FFCOMP || m.etype == FS_Q4RSCOMP);
    if (m.nen == 3)
        k_normals<3><<<nblk2(m.nnodes, 128), 128, 0, c->stream>>>(m, comp, cos_thr, cs, m.normals, m.valid);
    else
        k_normals<4><<<nblk2(m.nnodes, 128), 128, 0, c->stream>>>(m, comp, cos_thr, cs, m.normals, m.valid);
    FS_CUDA(c, cudaGetLastError());
    return round_normals(c);
}

// ---------------------------------------------------------------------------
// lumped mass
// ---------------------------------------------------------------------------
template <int NN>
__global__ void k_masses(const MeshDev m, double rho, bool comp, double *tmrm)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nelem) return;
    ElemIn<NN> in;
    for (int a = 0; a < NN; a++) {
        int node = m.conn[r * NN + a];
        for (int c = 0; c < 3; c++) in.X[a][c] = m.xyz[(int64_t)c * m.nnodes + node];
    }
    in.t = m.thick ? m.thick[r] : 0.0;
    const GroupConst *gc = comp ? &m.groups[m.group[r]] : nullptr;
    double tm, rm;
    lumped_mass<NN>(in, rho, comp, gc, tm, rm);
    tmrm[2 * r] = tm;
    tmrm[2 * r + 1] = rm;
}

int launch_masses(fs_ctx *c)
{
    MeshDev &m = c->mesh;
    FS_TRY(dalloc(c, &c->tmrm, (size_t)(2 * m.nelem)));
    if (m.nelem == 0) return FS_OK;
    bool comp = (m.etype == FS_T3FFCOMP || m.etype == FS_Q4RSCOMP);
    if (m.nen == 3)
        k_masses<3><<<nblk2(m.nelem, 128), 128, 0, c->stream>>>(m, c->params.rho, comp, c->tmrm);
    else
        k_masses<4><<<nblk2(m.nelem, 128), 128, 0, c->stream>>>(m, c->params.rho, comp, c->tmrm);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

// Diagonal mass values: node sums in assembly order.  `diag_pos` selects the
// destination: the diagonal pattern (value index d-1) or the position of the
// diagonal entry inside the full pattern.
__global__ void k_mass_assemble(const MeshDev m, const PatternDev P, int64_t n, const double *tmrm,
                                bool full_pattern, double *vals)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nnodes) return;
    double tsum = 0.0, rsum = 0.0;
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        int64_t rank = m.pair_e[p] >> 2;
        tsum += tmrm[2 * rank];
        rsum += tmrm[2 * rank + 1];
    }
    int self = -1;
    if (full_pattern) {
        int64_t off = P.nbr_off[r];
        int nn = (int)(P.nbr_off[r + 1] - off);
        int lo = 0, hi = nn - 1;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (P.nbr[off + mid] < r) lo = mid + 1; else hi = mid;
        }
        self = lo;
    }
    for (int k = 0; k < 6; k++) {
        int32_t d = m.dof[(int64_t)k * m.nnodes + r];
        if (d > n) continue;
        double v = k < 3 ? tsum : rsum;
        if (full_pattern) {
            int cp = P.colpos[P.nbr_off[r] * 6 + self * 6 + k];
            vals[P.rowptr[d - 1] + cp] = v;
        } else {
            vals[d - 1] = v;
        }
    }
}

int assemble_mass(fs_ctx *c, int assembler, int64_t n)
{
    MeshDev &m = c->mesh;
    PatternDev &P = c->pat;
    bool full = (assembler == FS_ASM_SPARSE);
    int64_t nnz = full ? P.nnz : n;
    if ((size_t)nnz > c->vals_cap || !c->vals) {
        FS_TRY(dalloc(c, &c->vals, (size_t)nnz));
        c->vals_cap = (size_t)nnz;
    }
    FS_CUDA(c, cudaMemsetAsync(c->vals, 0, sizeof(double) * std::max<int64_t>(nnz, 1), c->stream));
    if (m.nnodes)
        k_mass_assemble<<<nblk2(m.nnodes, 128), 128, 0, c->stream>>>(m, P, n, c->tmrm, full, c->vals);
    FS_CUDA(c, cudaGetLastError());
    c->mat_kind = 1;
    c->mat_n = n;
    if (full) {
        c->mat_rowptr = P.rowptr;
        c->mat_colidx = P.colidx;
        c->mat_nnz = P.nnz;
    } else {
        c->mat_rowptr = P.diag_rowptr;
        c->mat_colidx = P.diag_colidx;
        c->mat_nnz = n;
        if (assembler == FS_ASM_SPARSE_SYMM)
            return compact_zeros(c, n, P.diag_rowptr, P.diag_colidx, c->vals, n);
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // namespace fs

namespace fs {

// Element matrices of every element into a caller-chosen buffer `ke`
// (same layout as the context's own buffer); allocates nothing.
int launch_elements_to(fs_ctx *c, int precision, void *ke)
{
    if (c->mesh.nelem == 0) return FS_OK;
    return run_elements(c, precision, ke);
}


// ---------------------------------------------------------------------------
// tile-shape autotuner
// ---------------------------------------------------------------------------
// Candidates: elements per block of the element kernel (T3: 32, 64, 128;
// Q4: 8, 16, 32, as far as their shared memory fits in 227 KB) and warps
// per block of the gather (4, 8, 16).  Each candidate is timed on the
// context's own mesh with CUDA events (best of three launches), the element
// kernel first, then the gather on its output.  The choice is keyed on
// element family, precision, the average-K option and log2 of the element
// count, and kept for the whole process.  Tile shapes change only how
// elements and nodes are grouped into blocks, never the arithmetic of one
// element or one stored value, so every candidate gives bitwise the same
// matrix.
namespace {
struct TuneKey {
    int etype, precision, avgk, bucket;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(etype, precision, avgk, bucket) < std::tie(o.etype, o.precision, o.avgk, o.bucket);
    }
};
std::mutex g_tune_mu;
struct TuneVal {
    int epb, warps, once;
};
std::map<TuneKey, TuneVal> g_tune;
const size_t SMEM_MAX = 227 * 1024;
const int64_t TUNE_MIN_ELEMENTS = 4096;
}  // namespace

static int time_best(fs_ctx *c, int (*run)(fs_ctx *, int), int precision, float *best_ms)
{
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        FS_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
        FS_TRY(run(c, precision));
        FS_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
        FS_CUDA(c, cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        FS_CUDA(c, cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        best = ms < best ? ms : best;
    }
    *best_ms = best;
    return FS_OK;
}

static int run_elements_once(fs_ctx *c, int precision) { return launch_elements(c, precision); }
static int run_gather_once(fs_ctx *c, int precision) { return launch_gather(c, precision, c->vals); }

int autotune_shell(fs_ctx *c, int precision)
{
    if (c->tune.mode < 0) {
        const char *e = getenv("FLEXSHELL_AUTOTUNE");
        c->tune.mode = (e && e[0] == '0') ? 0 : 1;
    }
    const MeshDev &m = c->mesh;
    c->tune.from_tuner = false;
    if (c->tune.mode == 0 || c->tune.mode == 3 || m.nelem < TUNE_MIN_ELEMENTS) {
        c->tune.elem_epb = 0;
        c->tune.gather_warps = 0;
        c->tune.gather_once = c->tune.mode == 3 ? 0 : -1;
        return FS_OK;
    }
    const bool avgk = c->params.transv_shear_formulation == 1;
    int bucket = 0;
    while ((int64_t(1) << (bucket + 1)) <= m.nelem) bucket++;
    const TuneKey key{m.etype, precision, avgk ? 1 : 0, bucket};
    if (c->tune.mode == 1) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            c->tune.elem_epb = it->second.epb;
            c->tune.gather_warps = it->second.warps;
            c->tune.gather_once = it->second.once;
            c->tune.from_tuner = true;
            return FS_OK;
        }
    }
    const bool t3 = m.nen == 3;
    const int ecand[3] = {t3 ? 32 : 8, t3 ? 64 : 16, t3 ? 128 : 32};
    int best_e = 0;
    float best_ms = 1e30f;
    for (int epb : ecand) {
        const size_t smem = t3 ? t3_smem(precision, avgk, m.etype == FS_T3FFCOMP, epb)
                               : q4_smem(precision, m.etype == FS_Q4RSCOMP, epb);
        if (smem > SMEM_MAX) continue;
        c->tune.elem_epb = epb;
        float ms = 0.f;
        FS_TRY(time_best(c, run_elements_once, precision, &ms));
        if (ms < best_ms) {
            best_ms = ms;
            best_e = epb;
        }
    }
    c->tune.elem_epb = best_e;
    FS_TRY(launch_elements(c, precision));  // the gather candidates read these element matrices
    // gather: warps per block, and whether node-block pairs are summed once
    // (with transposed copies) or by both nodes; bitwise the same values
    int best_w = 0, best_o = 1;
    best_ms = 1e30f;
    for (int w : {4, 8, 16}) {
        if (gather_smem_bytes(precision, m.nen, w) > SMEM_MAX) continue;
        for (int once : {1, 0}) {
            c->tune.gather_warps = w;
            c->tune.gather_once = once;
            float ms = 0.f;
            FS_TRY(time_best(c, run_gather_once, precision, &ms));
            if (ms < best_ms) {
                best_ms = ms;
                best_w = w;
                best_o = once;
            }
        }
    }
    c->tune.gather_warps = best_w;
    c->tune.gather_once = best_o;
    c->tune.from_tuner = true;
    if (c->tune.mode == 2) c->tune.mode = 1;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = {best_e, best_w, best_o};
    return FS_OK;
}

}  // namespace fs

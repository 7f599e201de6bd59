// C ABI of the flexshell library (include/flexshell.h).
#include <string.h>

#include <algorithm>
#include <vector>

#include "fs_host_prep.h"
#include "fs_internal.cuh"

namespace fs {

int set_err(fs_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_check(fs_ctx *c, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return FS_OK;
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation)
        return set_err(c, FS_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    return set_err(c, FS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int ensure_scratch(fs_ctx *c, size_t bytes)
{
    if (bytes <= c->scratch_bytes && c->scratch) return FS_OK;
    // the scratch may be in use by queued work: wait before replacing it
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&c->scratch, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(c, FS_ERR_OOM, "scratch allocation failed");
    }
    c->scratch_bytes = bytes;
    return FS_OK;
}

int read_status(fs_ctx *c, int *bits)
{
    int h = 0;
    FS_CUDA(c, cudaMemcpyAsync(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (h) FS_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
    *bits = h;
    return FS_OK;
}

static void free_pattern(PatternDev &P)
{
    dfree(&P.nbr_off); dfree(&P.nbr); dfree(&P.pair_slots); dfree(&P.colpos); dfree(&P.colsrc); dfree(&P.rowlen);
    dfree(&P.sl_off); dfree(&P.sl_ent); dfree(&P.sl_mir); dfree(&P.lc);
    dfree(&P.rowptr); dfree(&P.colidx); dfree(&P.diag_rowptr); dfree(&P.diag_colidx);
    dfree(&P.tmp_cnt); dfree(&P.tmp_owner);
    P = PatternDev();
}

// invalidate the pattern (new mesh or dof numbering) keeping its buffers for
// the next build: no device free or allocation between assemblies
static void reset_pattern(PatternDev &P)
{
    P.n = -1;
    P.nnz = 0;
    P.maxlen = 0;
}

static void free_mesh(MeshDev &m)
{
    dfree(&m.xyz); dfree(&m.conn); dfree(&m.elem_of_rank); dfree(&m.dof); dfree(&m.thick);
    dfree(&m.group); dfree(&m.groups); dfree(&m.normals); dfree(&m.normals_f); dfree(&m.valid); dfree(&m.pp);
    dfree(&m.pair_e); dfree(&m.elem_pair);
    m = MeshDev();
}


__global__ void k_fill_d(int64_t n, double v, double *p)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_plus_one_i64(int64_t n, const int64_t *src, int64_t *dst)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i] + 1;
}

__global__ void k_plus_one_i32(int64_t n, const int32_t *src, int64_t *dst)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (int64_t)src[i] + 1;
}

// diagonal of a CSR matrix (sorted columns)
__global__ void k_extract_diag(int64_t n, const int64_t *rowptr, const int32_t *colidx, const double *vals,
                               double *diag)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t lo = rowptr[i], hi = rowptr[i + 1] - 1;
    double v = 0.0;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        int32_t cc = colidx[mid];
        if (cc == i) { v = vals[mid]; break; }
        if (cc < i) lo = mid + 1; else hi = mid - 1;
    }
    diag[i] = v;
}

static bool is_comp(int et) { return et == FS_T3FFCOMP || et == FS_Q4RSCOMP; }

int check_ready(fs_ctx *c, bool need_dofs)
{
    if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    if (c->mesh.etype == FS_COROTBEAM)
        return set_err(c, FS_ERR_UNSUPPORTED, "beam mesh: use the fs_beam_* entry points");
    if (!c->params_set) return set_err(c, FS_ERR_STATE, "no parameters: call fs_params_set first");
    if (need_dofs && !c->dofs_ready) return set_err(c, FS_ERR_STATE, "no dof numbering: call fs_dofs_set first");
    if (is_comp(c->mesh.etype) && !c->mesh.groups)
        return set_err(c, FS_ERR_STATE, "layered FEMM without layups: call fs_layups_set first");
    return FS_OK;
}

int check_last_stiffness(fs_ctx *c)
{
    if (!c->mat_rowptr || c->mat_kind != 0)
        return set_err(c, FS_ERR_STATE, "no stiffness: fs_stiffness must be the last matrix assembled");
    return FS_OK;
}

int status_to_code(fs_ctx *c, int bits)
{
    if (bits & DEV_SINGULAR) return set_err(c, FS_ERR_SINGULAR_METRIC, "Singular metric matrix in _gradN_e!");
    if (bits & DEV_NEG_DRILL) return set_err(c, FS_ERR_UNSUPPORTED, "negative drilling stiffness");
    if (bits) return set_err(c, FS_ERR_BAD_INPUT, "invalid input detected on the device");
    return FS_OK;
}

}  // namespace fs

using namespace fs;

static int apply_thickness(fs_ctx *c)
{
    MeshDev &m = c->mesh;
    if (!c->params_set || m.etype < 0) return FS_OK;
    if (!c->h_thickness.empty() && (int64_t)c->h_thickness.size() == m.nelem)
        return upload_by_rank<double>(c, c->h_thickness.data(), m.nelem, &m.thick);
    FS_TRY(dalloc(c, &m.thick, (size_t)m.nelem));
    if (m.nelem)
        k_fill_d<<<(unsigned)((m.nelem + 255) / 256), 256, 0, c->stream>>>(m.nelem, c->params.thickness, m.thick);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

static int apply_groups(fs_ctx *c)
{
    MeshDev &m = c->mesh;
    if (c->h_groups.empty() || m.etype < 0 || (int64_t)c->h_egroup.size() != m.nelem) return FS_OK;
    std::vector<GroupConst> gcs(c->h_groups.size());
    for (size_t g = 0; g < c->h_groups.size(); g++)
        if (prepare_group(c->h_groups[g], gcs[g]))
            return set_err(c, FS_ERR_BAD_INPUT, "layup stiffness [A B; B D] or H is not positive semi-definite");
    FS_TRY(dalloc(c, &m.groups, gcs.size()));
    FS_CUDA(c, cudaMemcpyAsync(m.groups, gcs.data(), sizeof(GroupConst) * gcs.size(), cudaMemcpyHostToDevice, c->stream));
    m.ngroups = (int)gcs.size();
    FS_TRY(upload_by_rank<int32_t>(c, c->h_egroup.data(), m.nelem, &m.group));
    return FS_OK;
}

extern "C" {

int fs_ctx_create(int device, fs_ctx **out)
{
    if (!out) return FS_ERR_BAD_INPUT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FS_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return FS_ERR_BAD_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return FS_ERR_CUDA;
    fs_ctx *c = new fs_ctx();
    c->device = device;
    for (int k = 0; k < 4; k++)
        if (cudaEventCreate(&c->ev[k]) != cudaSuccess) {
            cudaGetLastError();
            delete c;
            return FS_ERR_CUDA;
        }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return FS_ERR_CUDA;
    }
    noalloc_setup(c);
    *out = c;
    return FS_OK;
}

int fs_ctx_destroy(fs_ctx *c)
{
    if (!c) return FS_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_mesh(c->mesh);
    free_pattern(c->pat);
    free_beam(c);
    free_shift(c);
    if (c->ke) cudaFree(c->ke);
    dfree(&c->tmrm); dfree(&c->vals); dfree(&c->cmp_rowptr); dfree(&c->cmp_colidx); dfree(&c->cmp_vals);
    dfree(&c->stage64);
    if (c->scratch) cudaFree(c->scratch);
    auto &x = c->ex;
    if (x.exec) cudaGraphExecDestroy(x.exec);
    if (x.graph) cudaGraphDestroy(x.graph);
    dfree(&x.U); dfree(&x.V); dfree(&x.A); dfree(&x.F); dfree(&x.cU); dfree(&x.cV);
    dfree(&x.invMC); dfree(&x.C); dfree(&x.vals32); dfree(&x.U32);
    dfree(&x.blk); dfree(&x.res); dfree(&x.xp); dfree(&x.pad_of_dof);
    dfree(&x.Fmag); dfree(&x.mul); dfree(&x.step);
    cudaFree(c->d_status);
    for (int k = 0; k < 4; k++)
        if (c->ev[k]) cudaEventDestroy(c->ev[k]);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (int k = 0; k < 2; k++)
        if (c->copy_ev[k]) cudaEventDestroy(c->copy_ev[k]);
    cudaStreamDestroy(c->stream);
    delete c;
    return FS_OK;
}

int fs_last_error(const fs_ctx *c, char *buf, size_t len)
{
    if (!buf || len == 0) return FS_ERR_BAD_INPUT;
    const char *m = c ? c->err.c_str() : "no context";
    strncpy(buf, m, len - 1);
    buf[len - 1] = 0;
    return FS_OK;
}

int fs_stream(const fs_ctx *c, void **stream)
{
    if (!c || !stream) return FS_ERR_BAD_INPUT;
    *stream = (void *)c->stream;
    return FS_OK;
}

int fs_mesh_set(fs_ctx *c, int elem_type, int64_t nnodes, const double *xyz, int64_t nelem,
                const int64_t *conn, const int64_t *order, const int64_t *dofnums)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (elem_type < FS_T3FF || elem_type > FS_COROTBEAM) return set_err(c, FS_ERR_BAD_INPUT, "unknown element type");
    if (nnodes < 0 || nelem < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative size");
    if ((nnodes && !xyz) || (nelem && !conn))
        return set_err(c, FS_ERR_BAD_INPUT, "missing mesh array");
    if (nelem >= (1LL << 29) || nnodes >= (1LL << 31))
        return set_err(c, FS_ERR_UNSUPPORTED, "mesh too large (elements < 2^29, nodes < 2^31)");
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    free_mesh(c->mesh);
    reset_pattern(c->pat);
    c->mat_rowptr = nullptr;
    free_shift(c);  // a factor of the previous mesh's stiffness
    free_beam(c);
    c->batch = fs_ctx::Batch();
    c->normals_ready = false;
    end_explicit(c);
    MeshDev &m = c->mesh;
    m.etype = elem_type;
    m.nen = (elem_type == FS_T3FF || elem_type == FS_T3FFCOMP) ? 3 : (elem_type == FS_COROTBEAM ? 2 : 4);
    m.nnodes = nnodes;
    m.nelem = nelem;
    FS_TRY(dalloc(c, &m.xyz, (size_t)(3 * nnodes)));
    FS_TRY(dalloc(c, &m.conn, (size_t)(nelem * m.nen)));
    FS_TRY(dalloc(c, &m.elem_of_rank, (size_t)nelem));
    FS_TRY(dalloc(c, &m.dof, (size_t)(6 * nnodes)));
    FS_TRY(dalloc(c, &m.normals, (size_t)(3 * nnodes)));
    FS_TRY(dalloc(c, &m.normals_f, (size_t)(3 * nnodes)));
    FS_TRY(dalloc(c, &m.valid, (size_t)nnodes));
    // raw uploads share one staging allocation
    size_t nconn = (size_t)(nelem * m.nen), nord = order ? (size_t)nelem : 0;
    size_t ndof = dofnums ? (size_t)(6 * nnodes) : 0;
    FS_TRY(ensure_scratch(c, sizeof(int64_t) * (nconn + nord + ndof + 3)));
    int64_t *raw = (int64_t *)c->scratch;
    int64_t *d_conn = raw, *d_order = order ? raw + nconn : nullptr;
    int64_t *d_dof = dofnums ? raw + nconn + nord : nullptr;
    if (nnodes) FS_CUDA(c, cudaMemcpyAsync(m.xyz, xyz, sizeof(double) * 3 * nnodes, cudaMemcpyHostToDevice, c->stream));
    if (nconn) FS_CUDA(c, cudaMemcpyAsync(d_conn, conn, sizeof(int64_t) * nconn, cudaMemcpyHostToDevice, c->stream));
    if (nord) FS_CUDA(c, cudaMemcpyAsync(d_order, order, sizeof(int64_t) * nord, cudaMemcpyHostToDevice, c->stream));
    if (ndof) FS_CUDA(c, cudaMemcpyAsync(d_dof, dofnums, sizeof(int64_t) * ndof, cudaMemcpyHostToDevice, c->stream));
    // launch_prepare_mesh may reuse the scratch for its own temporaries only after
    // these kernels consumed the raw arrays (it synchronises inside)
    int st = launch_prepare_mesh(c, d_conn, d_order, d_dof);
    if (st != FS_OK) {
        free_mesh(c->mesh);
        return st;
    }
    st = build_adjacency(c);
    if (st != FS_OK) {
        free_mesh(c->mesh);
        return st;
    }
    c->dofs_ready = dofnums != nullptr;
    FS_TRY(apply_thickness(c));
    FS_TRY(apply_groups(c));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_geometry_set(fs_ctx *c, const double *xyz)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    if (c->mesh.nnodes && !xyz) return set_err(c, FS_ERR_BAD_INPUT, "missing geometry");
    if (c->mesh.nnodes)
        FS_CUDA(c, cudaMemcpyAsync(c->mesh.xyz, xyz, sizeof(double) * 3 * c->mesh.nnodes, cudaMemcpyHostToDevice,
                                   c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_dofs_set(fs_ctx *c, const int64_t *dofnums)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    MeshDev &m = c->mesh;
    if (m.nnodes && !dofnums) return set_err(c, FS_ERR_BAD_INPUT, "missing dof numbers");
    reset_pattern(c->pat);
    end_explicit(c);
    c->mat_rowptr = nullptr;
    free_shift(c);  // its band and size follow the previous numbering
    size_t ndof = (size_t)(6 * m.nnodes);
    FS_TRY(ensure_scratch(c, sizeof(int64_t) * (ndof + 1)));
    int64_t *raw = (int64_t *)c->scratch;
    if (ndof) FS_CUDA(c, cudaMemcpyAsync(raw, dofnums, sizeof(int64_t) * ndof, cudaMemcpyHostToDevice, c->stream));
    FS_TRY(launch_prepare_dofs(c, raw));
    c->dofs_ready = true;
    return FS_OK;
}

int fs_params_set(fs_ctx *c, const fs_shell_params *p, const double *thickness)
{
    if (!c || !p) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (p->transv_shear_formulation != 0 && p->transv_shear_formulation != 1)
        return set_err(c, FS_ERR_UNSUPPORTED, "transv_shear_formulation must be 0 (average B) or 1 (average K)");
    if (p->drilling_stiffness_scale < 0.0)
        return set_err(c, FS_ERR_UNSUPPORTED, "negative drilling_stiffness_scale");
    if (!(p->stab_c >= 0.0)) return set_err(c, FS_ERR_UNSUPPORTED, "stab_fun coefficient must be >= 0");
    MatConst mc;
    if (prepare_matconst(*p, mc))
        return set_err(c, FS_ERR_BAD_INPUT, "material stiffness Dps or Dt is not positive semi-definite");
    c->params = *p;
    c->mc = mc;
    c->params_set = true;
    c->h_thickness.clear();
    if (thickness) {
        if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "per-element thickness needs a mesh");
        c->h_thickness.assign(thickness, thickness + c->mesh.nelem);
    }
    FS_TRY(apply_thickness(c));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_layups_set(fs_ctx *c, int32_t ngroups, const fs_layup_group *groups, const int32_t *elem_group)
{
    if (!c || ngroups <= 0 || !groups) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    c->h_groups.assign(groups, groups + ngroups);
    c->h_egroup.assign((size_t)c->mesh.nelem, 0);
    if (elem_group) {
        for (int64_t e = 0; e < c->mesh.nelem; e++) {
            if (elem_group[e] < 0 || elem_group[e] >= ngroups)
                return set_err(c, FS_ERR_BAD_INPUT, "element layup group out of range");
            c->h_egroup[e] = elem_group[e];
        }
    }
    FS_TRY(apply_groups(c));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->normals_ready = false;
    return FS_OK;
}

int fs_normals_compute(fs_ctx *c)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c, false));
    FS_TRY(launch_normals(c));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->normals_ready = true;
    return FS_OK;
}

int fs_normals_compute_csys(fs_ctx *c, int kind, const double *params)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c, false));
    if (kind < FS_CSYS_ISOPARAMETRIC || kind > FS_CSYS_SPHERICAL)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown csys kind");
    if (kind != FS_CSYS_ISOPARAMETRIC && !params) return set_err(c, FS_ERR_BAD_INPUT, "missing csys parameters");
    if (kind != FS_CSYS_ISOPARAMETRIC && is_comp(c->mesh.etype))
        return set_err(c, FS_ERR_UNSUPPORTED, "layered FEMMs take their normals from the layup csys");
    FS_TRY(launch_normals(c, kind, params));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->normals_ready = true;
    return FS_OK;
}

int fs_normals_set(fs_ctx *c, const double *normals, const uint8_t *valid)
{
    if (!c || !normals || !valid) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    if (c->mesh.etype == FS_COROTBEAM)
        return set_err(c, FS_ERR_UNSUPPORTED, "beam mesh: beams have no shell normals");
    int64_t nn = c->mesh.nnodes;
    FS_CUDA(c, cudaMemcpyAsync(c->mesh.normals, normals, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, c->stream));
    FS_TRY(round_normals(c));
    FS_CUDA(c, cudaMemcpyAsync(c->mesh.valid, valid, nn, cudaMemcpyHostToDevice, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->normals_ready = true;
    return FS_OK;
}

int fs_normals_get(fs_ctx *c, double *normals, uint8_t *valid)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (!c->normals_ready) return set_err(c, FS_ERR_STATE, "normals not available: call fs_normals_compute");
    int64_t nn = c->mesh.nnodes;
    if (normals) FS_CUDA(c, cudaMemcpyAsync(normals, c->mesh.normals, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, c->stream));
    if (valid) FS_CUDA(c, cudaMemcpyAsync(valid, c->mesh.valid, nn, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // extern "C"

// Pattern (built on the first call for a matrix size), element kernel, CSR
// gather and the assembler's post-processing.  beam_which < 0: shell
// stiffness; else the beam matrix FS_BEAM_*.
int fs::assemble_matrix(fs_ctx *c, int precision, int assembler, int64_t nrows, int64_t *nnz_out, int beam_which,
                        int mass_type)
{
    end_explicit(c);  // the current matrix (and maybe the pattern) changes
    if (c->pat.n != nrows || !c->pat.rowptr) {
        FS_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
        FS_TRY(build_pattern(c, nrows));
        FS_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
        FS_CUDA(c, cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        c->t_symbolic_ms = ms;
    }
    PatternDev &P = c->pat;
    c->timed = false;
    size_t need = (size_t)std::max<int64_t>(P.nnz, nrows);
    if (need > c->vals_cap || !c->vals) {
        FS_TRY(dalloc(c, &c->vals, need));
        c->vals_cap = need;
    }
    if (beam_which < 0) FS_TRY(autotune_shell(c, precision));
    FS_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    FS_TRY(beam_which < 0 ? launch_elements(c, precision) : launch_beam_elements(c, beam_which, mass_type));
    FS_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
    FS_TRY(launch_gather(c, precision, c->vals));
    FS_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    FS_TRY(status_to_code(c, bits));
    c->timed = true;
    c->t_compact_ms = 0.0;
    c->mat_kind = (beam_which < 0 || beam_which == FS_BEAM_STIFFNESS) ? 0 : 2;
    c->mat_n = nrows;
    c->mat_rowptr = P.rowptr;
    c->mat_colidx = P.colidx;
    c->mat_nnz = P.nnz;
    if (assembler == FS_ASM_SPARSE_SYMM) {
        FS_TRY(compact_zeros(c, nrows, P.rowptr, P.colidx, c->vals, P.nnz));
        FS_CUDA(c, cudaEventRecord(c->ev[3], c->stream));
        FS_CUDA(c, cudaEventSynchronize(c->ev[3]));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        c->t_compact_ms = ms;
    } else if (assembler == FS_ASM_DIAG) {
        double *dg = nullptr;
        FS_TRY(dalloc(c, &dg, (size_t)nrows));
        if (nrows)
            k_extract_diag<<<(unsigned)((nrows + 255) / 256), 256, 0, c->stream>>>(nrows, P.rowptr, P.colidx, c->vals, dg);
        FS_CUDA(c, cudaMemcpyAsync(c->vals, dg, sizeof(double) * std::max<int64_t>(nrows, 0), cudaMemcpyDeviceToDevice, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(dg);
        c->mat_rowptr = P.diag_rowptr;
        c->mat_colidx = P.diag_colidx;
        c->mat_nnz = nrows;
    }
    if (nnz_out) *nnz_out = c->mat_nnz;
    return FS_OK;
}

extern "C" {

int fs_stiffness(fs_ctx *c, int precision, int assembler, int64_t nrows, int64_t *nnz_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype == FS_COROTBEAM)
        return set_err(c, FS_ERR_UNSUPPORTED, "beam mesh: use fs_beam_matrix (FS_BEAM_STIFFNESS)");
    FS_TRY(check_ready(c));
    if (precision != FS_FP64 && precision != FS_MIXED && precision != FS_MIXED_COMP)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown precision");
    if (assembler < FS_ASM_SPARSE || assembler > FS_ASM_DIAG) return set_err(c, FS_ERR_BAD_INPUT, "unknown assembler");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "associategeometry! has not been called (self._associatedgeometry == true)");
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative matrix size");
    return assemble_matrix(c, precision, assembler, nrows, nnz_out, -1, 0);
}

int fs_mass(fs_ctx *c, int assembler, int64_t nrows, int64_t *nnz_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c));
    if (assembler < FS_ASM_SPARSE || assembler > FS_ASM_DIAG) return set_err(c, FS_ERR_BAD_INPUT, "unknown assembler");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "associategeometry! has not been called (self._associatedgeometry == true)");
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative matrix size");
    end_explicit(c);  // the current matrix (and maybe the pattern) changes
    FS_TRY(build_pattern(c, nrows));
    FS_TRY(launch_masses(c));
    FS_TRY(assemble_mass(c, assembler, nrows));
    if (nnz_out) *nnz_out = c->mat_nnz;
    return FS_OK;
}

int fs_autotune(fs_ctx *c, int mode)
{
    if (!c) return FS_ERR_BAD_INPUT;
    if (mode < 0 || mode > 3) return set_err(c, FS_ERR_BAD_INPUT, "autotune mode must be 0, 1, 2 or 3");
    c->tune.mode = mode;
    return FS_OK;
}

int fs_tuning(const fs_ctx *c, int32_t *out)
{
    if (!c || !out) return FS_ERR_BAD_INPUT;
    out[0] = c->tune.elem_epb;
    out[1] = c->tune.gather_warps;
    out[2] = c->tune.from_tuner ? 1 : 0;
    return FS_OK;
}

int fs_tuning_ex(const fs_ctx *c, int32_t *out, int n)
{
    if (!c || (n > 0 && !out)) return FS_ERR_BAD_INPUT;
    const int32_t v[4] = {c->tune.elem_epb, c->tune.gather_warps, c->tune.from_tuner ? 1 : 0,
                          c->tune.gather_once != 0 ? 1 : 0};
    for (int k = 0; k < n && k < 4; k++) out[k] = v[k];
    return FS_OK;
}

int fs_timings(const fs_ctx *c, double *out, int n)
{
    if (!c || !out || n < 0) return FS_ERR_BAD_INPUT;
    double t[4] = {0, 0, c->t_symbolic_ms, c->t_compact_ms};
    if (c->timed) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        t[0] = a;
        t[1] = b;
    }
    for (int k = 0; k < n && k < 4; k++) out[k] = t[k];
    return FS_OK;
}

int fs_matrix_copy(fs_ctx *c, int64_t *colptr, int64_t *rowval, double *nzval)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (!c->mat_rowptr) return set_err(c, FS_ERR_STATE, "no matrix assembled");
    int64_t n = c->mat_n, nnz = c->mat_nnz;
    size_t need = (size_t)std::max<int64_t>(n + 1, nnz);
    if (need > c->stage_cap || !c->stage64) {
        FS_TRY(dalloc(c, &c->stage64, need));
        c->stage_cap = need;
    }
    if (colptr) {
        k_plus_one_i64<<<(unsigned)((n + 1 + 255) / 256), 256, 0, c->stream>>>(n + 1, c->mat_rowptr, c->stage64);
        FS_CUDA(c, cudaGetLastError());
        FS_CUDA(c, cudaMemcpyAsync(colptr, c->stage64, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (rowval && nnz) {
        k_plus_one_i32<<<(unsigned)((nnz + 255) / 256), 256, 0, c->stream>>>(nnz, c->mat_colidx, c->stage64);
        FS_CUDA(c, cudaGetLastError());
        FS_CUDA(c, cudaMemcpyAsync(rowval, c->stage64, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, c->stream));
    }
    if (nzval && nnz) FS_CUDA(c, cudaMemcpyAsync(nzval, c->vals, sizeof(double) * nnz, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_pattern(fs_ctx *c, int64_t nrows, int64_t *nnz_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c));
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative matrix size");
    if (c->pat.n != nrows || !c->pat.rowptr) {
        end_explicit(c);  // its captured steps read the pattern
        FS_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
        FS_TRY(build_pattern(c, nrows));
        FS_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
        FS_CUDA(c, cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        c->t_symbolic_ms = ms;
    }
    if (nnz_out) *nnz_out = c->pat.nnz;
    return FS_OK;
}

int fs_stiffness_copy(fs_ctx *c, int precision, int64_t nrows, int64_t *colptr, int64_t *rowval, double *nzval)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c));
    if (precision != FS_FP64 && precision != FS_MIXED && precision != FS_MIXED_COMP)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown precision");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "associategeometry! has not been called (self._associatedgeometry == true)");
    if (c->pat.n != nrows || !c->pat.rowptr) return set_err(c, FS_ERR_STATE, "no pattern of this size: call fs_pattern first");
    if (!colptr || (c->pat.nnz && (!rowval || !nzval))) return set_err(c, FS_ERR_BAD_INPUT, "missing output array");
    if (!c->copy_stream) {
        FS_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) FS_CUDA(c, cudaEventCreateWithFlags(&c->copy_ev[k], cudaEventDisableTiming));
    }
    const PatternDev &P = c->pat;
    const int64_t n = nrows, nnz = P.nnz;
    const size_t need = (size_t)(n + 1 + nnz);
    if (need > c->stage_cap || !c->stage64) {
        FS_TRY(dalloc(c, &c->stage64, need));
        c->stage_cap = need;
    }
    // the pattern (1-based) goes out on the copy stream while the kernels run;
    // the row indices are widened in chunks on the context stream, each
    // chunk's copy starting as soon as it is widened, so the host link is
    // busy from the first chunk on (a single widening pass ahead of one copy
    // left the link idle for its whole duration)
    int64_t *sp = c->stage64, *sr = c->stage64 + n + 1;
    k_plus_one_i64<<<(unsigned)((n + 1 + 255) / 256), 256, 0, c->stream>>>(n + 1, P.rowptr, sp);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaEventRecord(c->copy_ev[0], c->stream));
    FS_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->copy_ev[0], 0));
    FS_CUDA(c, cudaMemcpyAsync(colptr, sp, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, c->copy_stream));
    const int64_t CHUNK = (int64_t)1 << 22;  // 32 MB of 64-bit row indices
    for (int64_t k0 = 0; k0 < nnz; k0 += CHUNK) {
        const int64_t len = nnz - k0 < CHUNK ? nnz - k0 : CHUNK;
        k_plus_one_i32<<<(unsigned)((len + 255) / 256), 256, 0, c->stream>>>(len, P.colidx + k0, sr + k0);
        FS_CUDA(c, cudaGetLastError());
        // a wait takes the event's latest record at the time of the call, so
        // one event serves every chunk
        FS_CUDA(c, cudaEventRecord(c->copy_ev[0], c->stream));
        FS_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->copy_ev[0], 0));
        FS_CUDA(c, cudaMemcpyAsync(rowval + k0, sr + k0, sizeof(int64_t) * len, cudaMemcpyDeviceToHost,
                                   c->copy_stream));
    }
    FS_CUDA(c, cudaEventRecord(c->copy_ev[1], c->copy_stream));
    // values: element kernel and gather on the context stream, then their copy
    int64_t got = 0;
    const int st = assemble_matrix(c, precision, FS_ASM_SPARSE, nrows, &got, -1, 0);
    if (st != FS_OK) {
        cudaStreamSynchronize(c->copy_stream);
        return st;
    }
    if (nnz) FS_CUDA(c, cudaMemcpyAsync(nzval, c->vals, sizeof(double) * nnz, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamWaitEvent(c->stream, c->copy_ev[1], 0));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_matrix_device(fs_ctx *c, const int64_t **rowptr, const int32_t **colidx, const double **vals,
                     int64_t *nrows, int64_t *nnz)
{
    if (!c) return FS_ERR_BAD_INPUT;
    if (!c->mat_rowptr) return set_err(c, FS_ERR_STATE, "no matrix assembled");
    if (rowptr) *rowptr = c->mat_rowptr;
    if (colidx) *colidx = c->mat_colidx;
    if (vals) *vals = c->vals;
    if (nrows) *nrows = c->mat_n;
    if (nnz) *nnz = c->mat_nnz;
    return FS_OK;
}

int fs_element_matrices(fs_ctx *c, int precision, double *out)
{
    if (!c || !out) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c, false));
    if (precision != FS_FP64 && precision != FS_MIXED && precision != FS_MIXED_COMP)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown precision");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "associategeometry! has not been called (self._associatedgeometry == true)");
    FS_TRY(launch_elements(c, precision));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    FS_TRY(status_to_code(c, bits));
    MeshDev &m = c->mesh;
    int nen = m.nen, nd = 6 * nen;
    size_t per = (size_t)nd * nd;
    size_t stored = (size_t)n_upper_blocks(nen) * 36;
    std::vector<int32_t> eor((size_t)m.nelem);
    if (m.nelem)
        FS_CUDA(c, cudaMemcpy(eor.data(), m.elem_of_rank, sizeof(int32_t) * m.nelem, cudaMemcpyDeviceToHost));
    std::vector<double> kd;
    std::vector<float> kf;
    if (precision == FS_FP64) {
        kd.resize(stored * m.nelem);
        if (m.nelem) FS_CUDA(c, cudaMemcpy(kd.data(), c->ke, sizeof(double) * kd.size(), cudaMemcpyDeviceToHost));
    } else {
        // float entries, or float pairs (hi, lo) of the compensated path
        const size_t w = precision == FS_MIXED_COMP ? 2 : 1;
        kf.resize(w * stored * m.nelem);
        if (m.nelem) FS_CUDA(c, cudaMemcpy(kf.data(), c->ke, sizeof(float) * kf.size(), cudaMemcpyDeviceToHost));
    }
    for (int64_t r = 0; r < m.nelem; r++) {
        double *o = out + per * eor[r];
        for (int a = 0; a < nen; a++)
            for (int b = 0; b < nen; b++)
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++) {
                        size_t src = stored * r +
                                     (a <= b ? (size_t)ub(a, b, nen) * 36 + i * 6 + j : (size_t)ub(b, a, nen) * 36 + j * 6 + i);
                        double v = precision == FS_FP64         ? kd[src]
                                   : precision == FS_MIXED_COMP ? (double)kf[2 * src] + (double)kf[2 * src + 1]
                                                                : (double)kf[src];
                        o[(6 * a + i) + (size_t)nd * (6 * b + j)] = v;
                    }
    }
    return FS_OK;
}

int fs_element_masses(fs_ctx *c, double *out)
{
    if (!c || !out) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_ready(c, false));
    FS_TRY(launch_masses(c));
    MeshDev &m = c->mesh;
    std::vector<int32_t> eor((size_t)m.nelem);
    std::vector<double> t((size_t)(2 * m.nelem));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (m.nelem) {
        FS_CUDA(c, cudaMemcpy(eor.data(), m.elem_of_rank, sizeof(int32_t) * m.nelem, cudaMemcpyDeviceToHost));
        FS_CUDA(c, cudaMemcpy(t.data(), c->tmrm, sizeof(double) * t.size(), cudaMemcpyDeviceToHost));
    }
    for (int64_t r = 0; r < m.nelem; r++) {
        out[2 * eor[r]] = t[2 * r];
        out[2 * eor[r] + 1] = t[2 * r + 1];
    }
    return FS_OK;
}

// Laminate reduction, src/CompositeLayupModule.jl:246-330: plies from the
// bottom (z = -t/2 - offset) up; each ply's plane-stress matrix is rotated
// into the layup frame (T Dps T^T with T the stress transformation of
// -angle) and integrated through the thickness; H uses the rotated ply
// shear matrix with the Vinson-Sierakowski parabolic factor or a constant.
int fs_laminate(int32_t nplies, const double *ply_Dps, const double *ply_Dts, const double *ply_t,
                const double *ply_angle_deg, const double *ply_rho, double offset, int32_t shear_model,
                double tcf, fs_layup_group *out)
{
    if (nplies <= 0 || !ply_Dps || !ply_Dts || !ply_t || !ply_angle_deg || !out) return FS_ERR_BAD_INPUT;
    if (shear_model != 0 && shear_model != 1) return FS_ERR_BAD_INPUT;
    fs_layup_group g;
    memset(&g, 0, sizeof(g));
    double lt = 0.0;
    for (int k = 0; k < nplies; k++) lt += ply_t[k];
    double zs = -lt / 2 - offset;
    double md = 0.0, mi = 0.0;
    for (int k = 0; k < nplies; k++) {
        double ze = zs + ply_t[k];
        double ang = ply_angle_deg[k] / 180.0 * M_PI;
        // stress transformation ply -> layup: rotation by -angle
        double m = cos(-ang), n = sin(-ang);
        double T[3][3] = {{m * m, n * n, 2 * m * n}, {n * n, m * m, -2 * m * n}, {-m * n, m * n, m * m - n * n}};
        const double *D = ply_Dps + 9 * k;
        double TD[3][3], R[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int q = 0; q < 3; q++) s += T[i][q] * D[q + 3 * j];
                TD[i][j] = s;
            }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int q = 0; q < 3; q++) s += TD[i][q] * T[j][q];
                R[i][j] = s;
            }
        double dz1 = ze - zs, dz2 = (ze * ze - zs * zs) / 2, dz3 = (ze * ze * ze - zs * zs * zs) / 3;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                g.A[i + 3 * j] += dz1 * R[i][j];
                g.B[i + 3 * j] += dz2 * R[i][j];
                g.D[i + 3 * j] += dz3 * R[i][j];
            }
        // transverse shear: Tt^T Dts Tt with Tt = [c -s; s c] of +angle
        double c2 = cos(ang), s2 = sin(ang);
        double Tt[2][2] = {{c2, -s2}, {s2, c2}};
        const double *H = ply_Dts + 4 * k;
        double HT[2][2], Hr[2][2];
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) HT[i][j] = H[i + 2 * 0] * Tt[0][j] + H[i + 2 * 1] * Tt[1][j];
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) Hr[i][j] = Tt[0][i] * HT[0][j] + Tt[1][i] * HT[1][j];
        double f = shear_model == 0 ? 5.0 / 4 * (ze - zs - 4.0 / 3 * (ze * ze * ze - zs * zs * zs) / (lt * lt))
                                    : tcf * (ze - zs);
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) g.H[i + 2 * j] += f * Hr[i][j];
        double rho = ply_rho ? ply_rho[k] : 0.0;
        md += (ze - zs) * rho;
        mi += (ze * ze * ze - zs * zs * zs) * rho / 3;
        zs += ply_t[k];
    }
    g.csmat[0] = g.csmat[4] = g.csmat[8] = 1.0;
    g.thickness = lt;
    g.mass_density = md;
    g.moi_density = mi;
    *out = g;
    return FS_OK;
}

}  // extern "C"

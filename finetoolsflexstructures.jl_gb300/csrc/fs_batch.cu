// Batched assembly of several shell meshes (fs_batch_*).
//
// The meshes are fused into one mesh whose element list is the work-list of
// all meshes' elements (mesh by mesh) and whose dof numbering offsets each
// mesh's free rows: one element-kernel launch and one gather launch assemble
// all of them, however uneven their sizes.  The fused matrix is block
// diagonal; each mesh's matrix is the slice of its rows, with its columns
// shifted back.  Every value is computed by the same per-element arithmetic
// and summed over the same pairs in the same order as when the mesh is
// assembled alone, so the per-mesh results are bitwise those of fs_stiffness
// on that mesh.
#include <algorithm>
#include <vector>

#include "fs_internal.cuh"

namespace fs {

__global__ void k_slice_rowptr(int64_t n, const int64_t *rowptr, int64_t base, int64_t *out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) out[i] = rowptr[i] - base + 1;
}

__global__ void k_slice_colidx(int64_t nnz, const int32_t *colidx, int64_t coff, int64_t *out)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) out[k] = (int64_t)colidx[k] - coff + 1;
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_batch_set(fs_ctx *c, int elem_type, int32_t nmeshes, const int64_t *nnodes, const double *const *xyz,
                 const int64_t *nelem, const int64_t *const *conn, const int64_t *const *dofnums,
                 const int64_t *nrows, const double *thickness)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (elem_type != FS_T3FF && elem_type != FS_Q4RS)
        return set_err(c, FS_ERR_UNSUPPORTED, "batched assembly supports the homogeneous FS_T3FF and FS_Q4RS");
    if (!c->params_set) return set_err(c, FS_ERR_STATE, "no parameters: call fs_params_set first");
    if (nmeshes < 1 || !nnodes || !xyz || !nelem || !conn || !dofnums || !nrows || !thickness)
        return set_err(c, FS_ERR_BAD_INPUT, "missing batch array");
    const int nen = elem_type == FS_T3FF ? 3 : 4;
    int64_t NN = 0, NE = 0, N = 0;
    for (int i = 0; i < nmeshes; i++) {
        if (nnodes[i] < 0 || nelem[i] < 0 || nrows[i] < 0 || nrows[i] > 6 * nnodes[i])
            return set_err(c, FS_ERR_BAD_INPUT, "mesh sizes out of range");
        if ((nnodes[i] && (!xyz[i] || !dofnums[i])) || (nelem[i] && !conn[i]))
            return set_err(c, FS_ERR_BAD_INPUT, "missing mesh array");
        NN += nnodes[i];
        NE += nelem[i];
        N += nrows[i];
    }
    std::vector<double> X((size_t)(3 * NN));
    std::vector<int64_t> C((size_t)(nen * NE)), D((size_t)(6 * NN));
    std::vector<double> T((size_t)NE);
    std::vector<int64_t> roff((size_t)nmeshes + 1, 0);
    int64_t noff = 0, eoff = 0;
    for (int i = 0; i < nmeshes; i++) {
        const int64_t nn = nnodes[i], ne = nelem[i];
        for (int k = 0; k < 3; k++)
            for (int64_t a = 0; a < nn; a++) X[(size_t)(k * NN + noff + a)] = xyz[i][k * nn + a];
        for (int64_t e = 0; e < ne; e++)
            for (int a = 0; a < nen; a++) {
                const int64_t v = conn[i][e * nen + a];
                if (v < 1 || v > nn) return set_err(c, FS_ERR_BAD_INPUT, "connectivity refers to a node outside its mesh");
                C[(size_t)((eoff + e) * nen + a)] = v + noff;
            }
        // rows of this mesh go after the previous meshes' rows; its excluded
        // dofs (above nrows) stay excluded, above every row of the fused matrix
        for (int k = 0; k < 6; k++)
            for (int64_t a = 0; a < nn; a++) {
                const int64_t d = dofnums[i][k * nn + a];
                if (d < 1 || d > 0x3fffffffLL) return set_err(c, FS_ERR_BAD_INPUT, "dof numbers must be in 1..2^30-1");
                D[(size_t)(k * NN + noff + a)] = d <= nrows[i] ? d + roff[(size_t)i] : N + d;
            }
        for (int64_t e = 0; e < ne; e++) T[(size_t)(eoff + e)] = thickness[i];
        roff[(size_t)i + 1] = roff[(size_t)i] + nrows[i];
        noff += nn;
        eoff += ne;
    }
    if (N + 0x3fffffffLL > 0x7fffffffLL) return set_err(c, FS_ERR_UNSUPPORTED, "batch too large");
    const fs_shell_params p = c->params;
    FS_TRY(fs_mesh_set(c, elem_type, NN, X.data(), NE, C.data(), nullptr, D.data()));
    FS_TRY(fs_params_set(c, &p, T.data()));
    FS_TRY(fs_normals_compute(c));
    c->batch.active = true;
    c->batch.roff = roff;
    return FS_OK;
}

int fs_batch_stiffness(fs_ctx *c, int precision, int assembler, int64_t *nnz_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (!c->batch.active) return set_err(c, FS_ERR_STATE, "no batch: call fs_batch_set first");
    const std::vector<int64_t> &roff = c->batch.roff;
    const int nm = (int)roff.size() - 1;
    int64_t nnz = 0;
    FS_TRY(fs_stiffness(c, precision, assembler, roff[(size_t)nm], &nnz));
    if (nnz_out) {
        std::vector<int64_t> rp((size_t)nm + 1);
        for (int i = 0; i <= nm; i++)
            FS_CUDA(c, cudaMemcpyAsync(&rp[(size_t)i], c->mat_rowptr + roff[(size_t)i], sizeof(int64_t),
                                       cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int i = 0; i < nm; i++) nnz_out[i] = rp[(size_t)i + 1] - rp[(size_t)i];
    }
    return FS_OK;
}

int fs_batch_matrix_copy(fs_ctx *c, int32_t mesh, int64_t *colptr, int64_t *rowval, double *nzval)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (!c->batch.active || !c->mat_rowptr) return set_err(c, FS_ERR_STATE, "no batch matrix assembled");
    const std::vector<int64_t> &roff = c->batch.roff;
    // the row slices below index the current matrix: it must be the batch's
    // stiffness (a mass or another matrix size assembled since: refused)
    if (c->mat_kind != 0 || c->mat_n != roff.back())
        return set_err(c, FS_ERR_STATE, "the current matrix is not the batch's: call fs_batch_stiffness again");
    if (mesh < 0 || mesh >= (int32_t)roff.size() - 1) return set_err(c, FS_ERR_BAD_INPUT, "mesh index out of range");
    const int64_t r0 = roff[(size_t)mesh], n = roff[(size_t)mesh + 1] - r0;
    int64_t b[2];
    FS_CUDA(c, cudaMemcpyAsync(&b[0], c->mat_rowptr + r0, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaMemcpyAsync(&b[1], c->mat_rowptr + r0 + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    const int64_t base = b[0], nnz = b[1] - b[0];
    const size_t need = (size_t)std::max<int64_t>(n + 1, nnz);
    if (need > c->stage_cap || !c->stage64) {
        FS_TRY(dalloc(c, &c->stage64, need));
        c->stage_cap = need;
    }
    if (colptr) {
        k_slice_rowptr<<<(unsigned)((n + 1 + 255) / 256), 256, 0, c->stream>>>(n, c->mat_rowptr + r0, base, c->stage64);
        FS_CUDA(c, cudaGetLastError());
        FS_CUDA(c, cudaMemcpyAsync(colptr, c->stage64, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (rowval && nnz) {
        k_slice_colidx<<<(unsigned)((nnz + 255) / 256), 256, 0, c->stream>>>(nnz, c->mat_colidx + base, r0, c->stage64);
        FS_CUDA(c, cudaGetLastError());
        FS_CUDA(c, cudaMemcpyAsync(rowval, c->stage64, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, c->stream));
    }
    if (nzval && nnz)
        FS_CUDA(c, cudaMemcpyAsync(nzval, c->vals + base, sizeof(double) * nnz, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // extern "C"

// Stress resultants at the integration points of the homogeneous shells
// (inspectintegpoints of FEMMShellT3FF, src/FEMMShellT3FFModule.jl:850-962,
// and FEMMShellQ4RS, src/FEMMShellQ4RSModule.jl:1061-1170): one thread per
// integration point, double precision (the point math is in
// csrc/fs_elem_math.cuh).  The reference evaluates the points element by
// element and hands each to a Julia closure; here all points are evaluated in
// one launch and the host walks felist over the result.
#include "fs_elem_common.cuh"

namespace fs {

template <int NN>
__global__ void __launch_bounds__(128) k_resultants(const MeshDev m, const MatConst mc, const double *u, int quant,
                                                    const double *cs, int64_t ncs, double *out, int *status)
{
    constexpr int NPT = NN == 3 ? 1 : 4;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.nelem * NPT) return;
    const int64_t r = p / NPT;  // assembly rank
    const int j = (int)(p - r * NPT);
    ElemIn<NN> in;
    load_elem<NN>(m, r, in);
    double ue[6 * NN];
    for (int a = 0; a < NN; a++) {
        const int64_t node = m.conn[r * NN + a];
        for (int k = 0; k < 6; k++) ue[6 * a + k] = u[(int64_t)k * m.nnodes + node];
    }
    // output index: the point of the mesh element (element order)
    const int64_t q = (int64_t)m.elem_of_rank[r] * NPT + j;
    const double *c = ncs == 0 ? nullptr : (ncs == 1 ? cs : cs + 9 * q);
    double o[3];
    if constexpr (NN == 3) {
        t3_resultant(in, mc, ue, quant, c, o);
    } else {
        Q4Elem qe;
        q4_prepare(in, in.t, mc.stab_c, qe);
        if (q4_resultant(in, qe, j, mc, ue, quant, c, o)) {
            atomicOr(status, DEV_SINGULAR);
            o[0] = o[1] = o[2] = 0.0;
        }
    }
    for (int k = 0; k < 3; k++) out[3 * q + k] = o[k];
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_resultants(fs_ctx *c, int quantity, const double *U, const double *csmat, int64_t ncs, double *out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    const MeshDev &m = c->mesh;
    if (m.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    if (m.etype != FS_T3FF && m.etype != FS_Q4RS)
        return set_err(c, FS_ERR_UNSUPPORTED, "resultants are defined for the homogeneous shells (T3FF, Q4RS)");
    if (!c->params_set) return set_err(c, FS_ERR_STATE, "no parameters: call fs_params_set first");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "normals not available: call fs_normals_compute or fs_normals_set "
                                        "(associategeometry!)");
    if (quantity != FS_RES_MOMENT && quantity != FS_RES_SHEAR && quantity != FS_RES_MEMBRANE)
        return set_err(c, FS_ERR_BAD_INPUT, "quantity must be FS_RES_MOMENT, FS_RES_SHEAR or FS_RES_MEMBRANE");
    const int npt = m.etype == FS_T3FF ? 1 : 4;
    const int64_t npoints = m.nelem * npt;
    if (ncs != 0 && ncs != 1 && ncs != npoints)
        return set_err(c, FS_ERR_BAD_INPUT, "csmat: none (ncs = 0, the element frame), one 3x3 matrix "
                                            "(ncs = 1) or one per integration point");
    if (npoints == 0) return FS_OK;
    if (!U || (ncs && !csmat) || !out) return set_err(c, FS_ERR_BAD_INPUT, "missing array");
    const size_t nu = (size_t)m.nnodes * 6, nc = (size_t)ncs * 9, no = (size_t)npoints * 3;
    FS_TRY(ensure_scratch(c, sizeof(double) * (nu + nc + no)));
    double *du = (double *)c->scratch, *dc = du + nu, *dout = dc + nc;
    FS_CUDA(c, cudaMemcpyAsync(du, U, sizeof(double) * nu, cudaMemcpyHostToDevice, c->stream));
    if (nc) FS_CUDA(c, cudaMemcpyAsync(dc, csmat, sizeof(double) * nc, cudaMemcpyHostToDevice, c->stream));
    const unsigned grid = (unsigned)((npoints + 127) / 128);
    if (npt == 1)
        k_resultants<3><<<grid, 128, 0, c->stream>>>(m, c->mc, du, quantity, dc, ncs, dout, c->d_status);
    else
        k_resultants<4><<<grid, 128, 0, c->stream>>>(m, c->mc, du, quantity, dc, ncs, dout, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaMemcpyAsync(out, dout, sizeof(double) * no, cudaMemcpyDeviceToHost, c->stream));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    if (bits & DEV_SINGULAR) return set_err(c, FS_ERR_SINGULAR_METRIC, "Singular metric matrix");
    return FS_OK;
}

}  // extern "C"

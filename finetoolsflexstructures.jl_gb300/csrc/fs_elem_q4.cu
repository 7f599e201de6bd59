// Q4RS / Q4RSComp element kernel: four lanes per element, one per Gauss
// point (the element math is csrc/fs_elem_math.cuh).
#include "fs_elem_common.cuh"

namespace fs {

// The elements per block (the tuned tile) is a launch parameter (block size
// / 4): every tile runs the same compiled kernel and the same arithmetic.
template <class R, bool COMP, class S>
__global__ void __launch_bounds__(256) k_q4_elements(const MeshDev m, const MatConst mc, S *ke, int *status)
{
    constexpr int NR = 36, ND = 24, STRIDE = NR * ND + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int el = threadIdx.x >> 2, qp = threadIdx.x & 3;
    R *rows = reinterpret_cast<R *>(smem_raw) + el * STRIDE;
    int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 2) + el;
    const bool active = r < m.nelem;
    ElemIn<4> in;
    double tr[4] = {0, 0, 0, 0};
    // element constants computed once per element (by its first lane) and
    // shared with the other three lanes
    Q4Elem qe;
    if (active) {
        load_elem<4>(m, r, in);
        if (qp == 0) q4_prepare(in, COMP ? m.groups[in.group].thickness : in.t, mc.stab_c, qe);
    }
    {
        const int src = (threadIdx.x & 31) & ~3;
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) qe.Xr[a][c] = __shfl_sync(0xffffffffu, qe.Xr[a][c], src);
        qe.stab = __shfl_sync(0xffffffffu, qe.stab, src);
        if constexpr (sizeof(R) == 4) {
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int c = 0; c < 3; c++) qe.Xf[a][c] = __shfl_sync(0xffffffffu, qe.Xf[a][c], src);
        }
    }
    if (active) {
        const GroupConst *gc = COMP ? &m.groups[in.group] : nullptr;
        int st = q4_point_rows<R, COMP>(in, qe, qp, mc, gc, rows + qp * 8 * ND, ND, tr);
        if (st) {
            atomicOr(status, DEV_SINGULAR);
            for (int k = 0; k < 4; k++) tr[k] = 0.0;
        }
    }
    // sum the drilling traces of the four quadrature points (lanes 4el..4el+3)
#pragma unroll
    for (int k = 0; k < 4; k++) {
        tr[k] += __shfl_xor_sync(0xffffffffu, tr[k], 1);
        tr[k] += __shfl_xor_sync(0xffffffffu, tr[k], 2);
    }
    if (active && qp == 0) q4_drill_rows<R>(in, tr, mc.drill_scale, rows + 32 * ND, ND);
    __syncwarp();
    if (!active) return;
    S *out = ke + r * (10 * 36);
    // ten upper node blocks shared by the four lanes of the element
    for (int bi = qp; bi < 10; bi += 4) {
        int a = bi < 4 ? 0 : (bi < 7 ? 1 : (bi < 9 ? 2 : 3));
        int b = a + (bi - (a == 0 ? 0 : (a == 1 ? 4 : (a == 2 ? 7 : 9))));
        constexpr bool PAIR = sizeof(S) == 8 && sizeof(R) == 4;
        BlockAcc<R, PAIR> acc;
        acc.zero();
        if constexpr (!COMP) {
            // homogeneous: per Gauss point 3 membrane rows (translations only)
            // and 5 bending/shear rows; then one drilling row per node
#pragma unroll 1
            for (int j = 0; j < 4; j++) {
                gram_rows<0, 3, 0, 3>(acc, rows, ND, 8 * j, 8 * j + 3, a, b);
                gram_rows<0, 6, 0, 6>(acc, rows, ND, 8 * j + 3, 8 * j + 8, a, b);
            }
            if (a == b) gram_rows<3, 6, 3, 6>(acc, rows, ND, 32 + a, 33 + a, a, b);
        } else {
            gram_rows<0, 6, 0, 6>(acc, rows, ND, 0, NR, a, b);
        }
        acc.store(out + ub(a, b, 4) * 36);
    }
}

template <class R, bool COMP, class S = R>
static int run_q4(fs_ctx *c, S *ke)
{
    int epb = c->tune.elem_epb;
    if (epb != 16 && !(epb == 64 && sizeof(R) == 4)) epb = 32;
    const size_t smem = q4_smem(sizeof(R) == 8 ? FS_FP64 : FS_MIXED, epb);
    auto kern = k_q4_elements<R, COMP, S>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(c->mesh.nelem, epb), epb * 4, smem, c->stream>>>(c->mesh, c->mc, ke, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

// every Q4 variant: row precision, storage, layered
int run_q4_any(fs_ctx *c, int precision, void *ke)
{
    const bool comp = c->mesh.etype == FS_Q4RSCOMP;
    if (precision == FS_FP64) {
        double *k = (double *)ke;
        return comp ? run_q4<double, true>(c, k) : run_q4<double, false>(c, k);
    }
    if (precision == FS_MIXED_COMP) {
        float2 *k = (float2 *)ke;
        return comp ? run_q4<float, true>(c, k) : run_q4<float, false>(c, k);
    }
    float *k = (float *)ke;
    return comp ? run_q4<float, true>(c, k) : run_q4<float, false>(c, k);
}

}  // namespace fs

// T3FF / T3FFComp element kernel: one thread per element (the element
// math is csrc/fs_elem_math.cuh, the block stores csrc/fs_elem_common.cuh).
#include "fs_elem_common.cuh"

namespace fs {

// The elements per block (the tuned tile) is the block size, a launch
// parameter: every tile runs the same compiled kernel, so the tile never
// changes the arithmetic of an element (compiled variants could contract
// products and sums into FMAs differently).
// Resident blocks of 128 threads asked of the compiler (the register budget
// per thread).  Float rows stored as floats: 4 (128 registers) for
// homogeneous elements, whose occupancy is otherwise held by registers, 3
// (170) for the others.  Float rows stored as float pairs (Dot2 accumulators,
// 72 registers): 3 for homogeneous elements (shared memory allows 3 of the
// 128-element tiles), 2 (255) for the others.  Double rows: 2.
template <class R, bool COMP, bool AVGK, class S> struct T3MinBlocks {
    static constexpr bool dense = COMP || AVGK;
    static constexpr int value = sizeof(R) == 8 ? 2 : (sizeof(S) == 8 ? (dense ? 2 : 3) : (dense ? 3 : 4));
};

template <class R, bool COMP, bool AVGK, class S>
__global__ void __launch_bounds__(128, (T3MinBlocks<R, COMP, AVGK, S>::value))
    k_t3_elements(const MeshDev m, const MatConst mc, S *ke, int *status)
{
    constexpr int NR = T3Rows<AVGK>::N, NS = T3Rows<AVGK>::NS;
    constexpr int ND = 18;
    // homogeneous elements: the compact rows (126 values instead of 198);
    // layered ones: dense rows.  An odd stride keeps the threads' rows in
    // distinct shared-memory banks.
    constexpr int STRIDE = COMP ? NR * ND + 1 : CompactRows<3, NS>::SIZE + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *rows = reinterpret_cast<R *>(smem_raw) + threadIdx.x * STRIDE;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nelem) return;
    ElemIn<3> in;
    load_elem<3>(m, r, in);
    const GroupConst *gc = COMP ? &m.groups[in.group] : nullptr;
    int st = t3_rows<R, COMP, AVGK, !COMP>(in, mc, gc, rows, ND);
    if (st) atomicOr(status, DEV_NEG_DRILL);
    if constexpr (COMP)
        write_blocks<R, S, 3, false>(rows, NR, ke + r * (6 * 36));
    else
        write_blocks_compact<R, S, 3, NS>(rows, ke + r * (6 * 36));
}

template <class R, bool COMP, bool AVGK, class S = R>
static int run_t3(fs_ctx *c, S *ke)
{
    int epb = c->tune.elem_epb;
    if (epb <= 0) epb = (sizeof(R) == 8 && AVGK) ? 64 : 128;
    if (epb != 32 && epb != 64) epb = 128;
    if (sizeof(R) == 8 && AVGK && epb > 64) epb = 64;  // shared memory of the double average-K rows
    const size_t smem = t3_smem(sizeof(R) == 8 ? FS_FP64 : FS_MIXED, AVGK, COMP, epb);
    auto kern = k_t3_elements<R, COMP, AVGK, S>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(c->mesh.nelem, epb), epb, smem, c->stream>>>(c->mesh, c->mc, ke, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

// every T3 variant: row precision, storage, layered, average-K
int run_t3_any(fs_ctx *c, int precision, void *ke)
{
    const bool comp = c->mesh.etype == FS_T3FFCOMP;
    const bool avgk = c->params.transv_shear_formulation == 1;
    if (precision == FS_FP64) {
        double *k = (double *)ke;
        if (comp) return avgk ? run_t3<double, true, true>(c, k) : run_t3<double, true, false>(c, k);
        return avgk ? run_t3<double, false, true>(c, k) : run_t3<double, false, false>(c, k);
    }
    if (precision == FS_MIXED_COMP) {
        float2 *k = (float2 *)ke;
        if (comp) return avgk ? run_t3<float, true, true>(c, k) : run_t3<float, true, false>(c, k);
        return avgk ? run_t3<float, false, true>(c, k) : run_t3<float, false, false>(c, k);
    }
    float *k = (float *)ke;
    if (comp) return avgk ? run_t3<float, true, true>(c, k) : run_t3<float, true, false>(c, k);
    return avgk ? run_t3<float, false, true>(c, k) : run_t3<float, false, false>(c, k);
}

}  // namespace fs

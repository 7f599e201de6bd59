// Q4RS / Q4RSComp element kernel: four lanes per element, one per Gauss
// point (the element math is csrc/fs_elem_math.cuh).
//
// Each element's inputs (nodes, normals, flags, thickness) and its
// centroid-relative coordinates are staged in shared memory, one node per
// lane, and read from there by the four points: no lane holds the whole
// element in registers.  The element-level double work (centroid,
// stabilisation factor, drilling factor) is split over the four lanes by
// node where it is node-wise.  Homogeneous elements keep their rows in the
// compact layout (Q4Compact: membrane rows on the translations, drilling rows
// on one node's rotations), layered ones in the dense 36 x 24 layout.
#include "fs_elem_common.cuh"

namespace fs {

// per-element staging area (shared memory)
struct Q4Stage {
    ElemIn<4> in;
    Q4Elem qe;
};

// row values (R units) one element keeps in shared memory, with one of
// padding (an odd stride spreads the elements over the banks)
__host__ __device__ constexpr int q4_row_values(bool layered) { return layered ? 36 * 24 + 1 : Q4Compact::SIZE + 1; }

size_t q4_smem(int precision, bool layered, int epb)
{
    const size_t rv = (size_t)q4_row_values(layered) * (precision == FS_FP64 ? 8 : 4);
    return (size_t)epb * (sizeof(Q4Stage) + ((rv + 7) & ~(size_t)7));
}

// Shared memory (about 3 KB per float homogeneous element, 4-7 KB for the
// others) bounds the resident elements of an SM to 76 or fewer, 304 threads:
// the register budget of 255 per thread costs no occupancy.

// The elements per block (the tuned tile) is a launch parameter (block size
// / 4): every tile runs the same compiled kernel and the same arithmetic.
template <class R, bool COMP, class S>
__global__ void __launch_bounds__(128, 2) k_q4_elements(const MeshDev m, const MatConst mc, S *ke, int *status)
{
    constexpr int ND = 24;
    constexpr int RV = q4_row_values(COMP);
    constexpr size_t RB = ((size_t)RV * sizeof(R) + 7) & ~(size_t)7;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int epb = blockDim.x >> 2;
    const int el = threadIdx.x >> 2, qp = threadIdx.x & 3;
    Q4Stage &sg = reinterpret_cast<Q4Stage *>(smem_raw)[el];
    R *rows = reinterpret_cast<R *>(smem_raw + (size_t)epb * sizeof(Q4Stage) + (size_t)el * RB);
    const int64_t r = (int64_t)blockIdx.x * epb + el;
    const bool active = r < m.nelem;
    const int src = (threadIdx.x & 31) & ~3;  // the element's first lane
    // --- stage the element: lane qp loads node qp ---
    double Xa[3] = {0, 0, 0};
    if (active) {
        const int node = m.conn[r * 4 + qp];
        for (int c = 0; c < 3; c++) {
            Xa[c] = m.xyz[(int64_t)c * m.nnodes + node];
            sg.in.X[qp][c] = Xa[c];
            sg.in.nrm[qp][c] = m.normals[(int64_t)c * m.nnodes + node];
            sg.in.nrmf[qp][c] = m.normals_f[(int64_t)c * m.nnodes + node];
        }
        sg.in.valid[qp] = m.valid[node] != 0;
        if (qp == 0) {
            sg.in.t = m.thick ? m.thick[r] : 0.0;
            sg.in.group = m.group ? m.group[r] : 0;
        }
    }
    __syncwarp();
    // --- centroid-relative coordinates and the stabilisation factor
    //     (q4_prepare, split by node: the same operations in the same order) ---
    double mxd = 0.0;
    if (active) {
        double cen[3] = {0, 0, 0};
        for (int a = 0; a < 4; a++)
            for (int c = 0; c < 3; c++) cen[c] += sg.in.X[a][c];
        for (int c = 0; c < 3; c++) {
            cen[c] /= 4;
            sg.qe.Xr[qp][c] = Xa[c] - cen[c];
            sg.qe.Xf[qp][c] = (float)sg.qe.Xr[qp][c];
        }
        if (qp > 0) {
            const double dx = Xa[0] - sg.in.X[0][0], dy = Xa[1] - sg.in.X[0][1], dz = Xa[2] - sg.in.X[0][2];
            mxd = dx * dx + dy * dy + dz * dz;
        }
    }
    // the largest of the element's three distances (exact in any order)
    {
        const double o1 = __shfl_xor_sync(0xffffffffu, mxd, 1);
        mxd = o1 > mxd ? o1 : mxd;
        const double o2 = __shfl_xor_sync(0xffffffffu, mxd, 2);
        mxd = o2 > mxd ? o2 : mxd;
    }
    if (active && qp == 0) {
        const double t = COMP ? m.groups[sg.in.group].thickness : sg.in.t;
        sg.qe.stab = t * t / (t * t + mc.stab_c * mxd);
    }
    __syncwarp();
    // --- rows of this lane's quadrature point ---
    double tr[4] = {0, 0, 0, 0};
    if (active) {
        const GroupConst *gc = COMP ? &m.groups[sg.in.group] : nullptr;
        // FS_MIXED (float rows stored as floats): the points' tangents and
        // frames in float; the compensated mode keeps them double
        constexpr bool FFRAME = sizeof(R) == 4 && sizeof(S) == 4;
        int st;
        if constexpr (COMP)
            st = q4_point_rows<R, true, false, FFRAME>(sg.in, sg.qe, qp, mc, gc, rows + qp * 8 * ND, ND, tr);
        else
            st = q4_point_rows<R, false, true, FFRAME>(sg.in, sg.qe, qp, mc, gc, rows + qp * Q4Compact::GP, 0, tr);
        if (st) {
            atomicOr(status, DEV_SINGULAR);
            for (int k = 0; k < 4; k++) tr[k] = 0.0;
        }
    }
    constexpr bool FFRAME = sizeof(R) == 4 && sizeof(S) == 4;
    if constexpr (FFRAME) {
        // FS_MIXED: the drilling factor in float (q4_drill_rows_f), the
        // traces summed over the four points by shuffles
        float trf[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            trf[k] = (float)tr[k];
            trf[k] += __shfl_xor_sync(0xffffffffu, trf[k], 1);
            trf[k] += __shfl_xor_sync(0xffffffffu, trf[k], 2);
        }
        bool use = false;
        if (active) {
            const float *nv = sg.in.nrmf[qp];
            use = sg.in.valid[qp] && (dot3(nv, nv) != 0.f);
        }
        const unsigned um = __ballot_sync(0xffffffffu, use) >> src;
        if (active) {
            float sum = 0.f;
            int cnt = 0;
            for (int k = 0; k < 4; k++)
                if ((um >> k) & 1u) {
                    const float v = trf[k] * 0.5f;
                    sum += v > 0.f ? v : 0.f;
                    cnt++;
                }
            const float kavg = (cnt ? sum / (float)cnt : 0.f) * (float)mc.drill_scale;
            const float sk = kavg > 0.f ? sqrtf(kavg) : 0.f;
            R *o = rows + Q4Compact::DR + 3 * qp;
            if constexpr (COMP) o = rows + (32 + qp) * ND;
            if constexpr (COMP)
                for (int q = 0; q < 24; q++) o[q] = 0;
            R *oc = COMP ? o + 6 * qp + 3 : o;
            for (int c = 0; c < 3; c++) oc[c] = (use && kavg != 0.f) ? (R)(sk * sg.in.nrmf[qp][c]) : (R)0;
        }
    } else {
    // sum the drilling traces of the four quadrature points (lanes 4el..4el+3)
#pragma unroll
    for (int k = 0; k < 4; k++) {
        tr[k] += __shfl_xor_sync(0xffffffffu, tr[k], 1);
        tr[k] += __shfl_xor_sync(0xffffffffu, tr[k], 2);
    }
    // --- drilling rows (q4_drill_rows, node qp on lane qp) ---
    bool use = false;
    if (active) {
        const double *nv = sg.in.nrm[qp];
        use = sg.in.valid[qp] && (dot3(nv, nv) != 0.0);  // sqrt(x) != 0 exactly when x != 0
    }
    const unsigned um = __ballot_sync(0xffffffffu, use) >> src;
    if (active) {
        double sum = 0.0;
        int cnt = 0;
        for (int k = 0; k < 4; k++)
            if ((um >> k) & 1u) {
                const double v = tr[k] / 2.0;
                sum += v > 0.0 ? v : 0.0;
                cnt++;
            }
        const double kavg = (cnt ? sum / cnt : 0.0) * mc.drill_scale;
        const double sk = kavg > 0.0 ? sqrt(kavg) : 0.0;
        if constexpr (COMP) {
            R *o = rows + (32 + qp) * ND;
            for (int q = 0; q < 24; q++) o[q] = 0;
            if (use && kavg != 0.0)
                for (int c = 0; c < 3; c++) o[6 * qp + 3 + c] = (R)(sk * sg.in.nrm[qp][c]);
        } else {
            R *o = rows + Q4Compact::DR + 3 * qp;
            for (int c = 0; c < 3; c++) o[c] = (use && kavg != 0.0) ? (R)(sk * sg.in.nrm[qp][c]) : (R)0;
        }
    }
    }
    __syncwarp();
    if (!active) return;
    S *out = ke + r * (10 * 36);
    constexpr bool PAIR = sizeof(S) == 8 && sizeof(R) == 4;
    // The element's ten upper node blocks over its four lanes, every lane
    // running the same code at each step: first the diagonal block (qp, qp)
    // (its upper triangle), then the six off-diagonal blocks as twelve
    // half-blocks (rows 0-2 of each, then rows 3-5), three per lane.
    // Homogeneous elements: per Gauss point 3 membrane rows (translations
    // only, so rows 0-2 of a block) and 5 bending/shear rows; then one
    // drilling row per node (diagonal blocks only) -- the products and their
    // order of the dense layout.
    {
        const int a = qp;
        BlockAcc<R, PAIR> acc;
        acc.zero();
        if constexpr (!COMP) {
#pragma unroll 1
            for (int j = 0; j < 4; j++) {
                const R *gpb = rows + j * Q4Compact::GP;
                gram_rows_c<0, 3, 0, 3, Q4Compact::MS, 3, 0, true>(acc, gpb, 0, 3, a, a);
                gram_rows_c<0, 6, 0, 6, Q4Compact::BSS, 6, 0, true>(acc, gpb + Q4Compact::BS, 0, 5, a, a);
            }
            gram_rows_c<3, 6, 3, 6, 3, 0, 3, true>(acc, rows + Q4Compact::DR + 3 * a, 0, 1, a, a);
        } else {
            gram_rows<0, 6, 0, 6, true>(acc, rows, ND, 0, 36, a, a);
        }
        acc.template store<true>(out + ub(a, a, 4) * 36);
    }
#pragma unroll 1
    for (int t = 0; t < 3; t++) {
        const int u = qp + 4 * t, ob = u < 6 ? u : u - 6, i0 = u < 6 ? 0 : 3;
        // off-diagonal block ob: (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
        const int a = ob < 3 ? 0 : (ob < 5 ? 1 : 2);
        const int b = ob < 3 ? ob + 1 : (ob < 5 ? ob - 1 : 3);
        BlockAcc<R, PAIR, 3> acc;
        acc.zero();
        if constexpr (!COMP) {
#pragma unroll 1
            for (int j = 0; j < 4; j++) {
                const R *gpb = rows + j * Q4Compact::GP;
                if (i0 == 0) gram_rows_c<0, 3, 0, 3, Q4Compact::MS, 3, 0>(acc, gpb, 0, 3, a, b);
                gram_rows_h<0, 6, Q4Compact::BSS, 6>(acc, gpb + Q4Compact::BS, 0, 5, a, b, i0);
            }
        } else {
            gram_rows_h<0, 6, ND, 6>(acc, rows, 0, 36, a, b, i0);
        }
        acc.store(out + ub(a, b, 4) * 36 + 6 * i0);
    }
}

template <class R, bool COMP, class S = R>
static int run_q4(fs_ctx *c, S *ke)
{
    int epb = c->tune.elem_epb;
    if (epb != 8 && epb != 16 && epb != 32) epb = 16;
    const int prec = sizeof(R) == 8 ? FS_FP64 : FS_MIXED;
    while (epb > 16 && q4_smem(prec, COMP, epb) > 227 * 1024) epb /= 2;
    const size_t smem = q4_smem(prec, COMP, epb);
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

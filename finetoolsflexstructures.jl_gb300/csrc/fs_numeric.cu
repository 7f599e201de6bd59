// Numeric phase: nodal normals, element matrices, the deterministic CSR
// value gather and the lumped mass.
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

#include "fs_internal.cuh"

namespace fs {

static unsigned nblk2(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

template <int NN>
__device__ __forceinline__ void load_elem(const MeshDev &m, int64_t r, ElemIn<NN> &in)
{
    for (int a = 0; a < NN; a++) {
        int node = m.conn[r * NN + a];
        for (int c = 0; c < 3; c++) {
            in.X[a][c] = m.xyz[(int64_t)c * m.nnodes + node];
            in.nrm[a][c] = m.normals[(int64_t)c * m.nnodes + node];
        }
        in.valid[a] = m.valid[node] != 0;
    }
    in.t = m.thick ? m.thick[r] : 0.0;
    in.group = m.group ? m.group[r] : 0;
}

// ---------------------------------------------------------------------------
// element kernels
// ---------------------------------------------------------------------------
// 36 contiguous values of a 6x6 block (16-byte aligned) as 16-byte stores;
// `transpose` writes acc^T.
template <class R>
__device__ __forceinline__ void store_block(R *o, const R (&acc)[6][6], bool transpose)
{
    constexpr int V = 16 / sizeof(R);
    R buf[36];
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = 0; j < 6; j++) buf[i * 6 + j] = transpose ? acc[j][i] : acc[i][j];
    if (V == 4) {
        float4 *o4 = reinterpret_cast<float4 *>(o);
#pragma unroll
        for (int q = 0; q < 9; q++)
            o4[q] = make_float4((float)buf[4 * q], (float)buf[4 * q + 1], (float)buf[4 * q + 2], (float)buf[4 * q + 3]);
    } else {
        double2 *o2 = reinterpret_cast<double2 *>(o);
#pragma unroll
        for (int q = 0; q < 18; q++) o2[q] = make_double2((double)buf[2 * q], (double)buf[2 * q + 1]);
    }
}

template <class R, int NN>
__device__ __forceinline__ void write_blocks(const R *rows, int nrows, R *out)
{
    const int ND = 6 * NN;
    for (int a = 0; a < NN; a++)
        for (int b = a; b < NN; b++) {
            R acc[6][6];
#pragma unroll
            for (int i = 0; i < 6; i++)
#pragma unroll
                for (int j = 0; j < 6; j++) acc[i][j] = 0;
            for (int rho = 0; rho < nrows; rho++) {
                const R *rr = rows + rho * ND;
                R ra[6], rb[6];
#pragma unroll
                for (int i = 0; i < 6; i++) {
                    ra[i] = rr[6 * a + i];
                    rb[i] = rr[6 * b + i];
                }
#pragma unroll
                for (int i = 0; i < 6; i++)
#pragma unroll
                    for (int j = 0; j < 6; j++) acc[i][j] += ra[i] * rb[j];
            }
            store_block<R>(out + ub(a, b, NN) * 36, acc, false);
        }
}

template <class R, bool COMP, bool AVGK, int EPB>
__global__ void __launch_bounds__(EPB) k_t3_elements(const MeshDev m, const MatConst mc, R *ke, int *status)
{
    constexpr int NR = T3Rows<AVGK>::N;
    constexpr int ND = 18;
    constexpr int STRIDE = NR * ND + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *rows = reinterpret_cast<R *>(smem_raw) + threadIdx.x * STRIDE;
    int64_t r = (int64_t)blockIdx.x * EPB + threadIdx.x;
    if (r >= m.nelem) return;
    ElemIn<3> in;
    load_elem<3>(m, r, in);
    const GroupConst *gc = COMP ? &m.groups[in.group] : nullptr;
    int st = t3_rows<R, COMP, AVGK>(in, mc, gc, rows, ND);
    if (st) atomicOr(status, DEV_NEG_DRILL);
    write_blocks<R, 3>(rows, NR, ke + r * (6 * 36));
}

template <class R, bool COMP, int EPB>
__global__ void __launch_bounds__(EPB * 4) k_q4_elements(const MeshDev m, const MatConst mc, R *ke, int *status)
{
    constexpr int NR = 36, ND = 24, STRIDE = NR * ND + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int el = threadIdx.x >> 2, qp = threadIdx.x & 3;
    R *rows = reinterpret_cast<R *>(smem_raw) + el * STRIDE;
    int64_t r = (int64_t)blockIdx.x * EPB + el;
    const bool active = r < m.nelem;
    ElemIn<4> in;
    double tr[4] = {0, 0, 0, 0};
    if (active) {
        load_elem<4>(m, r, in);
        const GroupConst *gc = COMP ? &m.groups[in.group] : nullptr;
        Q4Elem qe;
        q4_prepare(in, qe);
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
    R *out = ke + r * (10 * 36);
    // ten upper node blocks shared by the four lanes of the element
    for (int bi = qp; bi < 10; bi += 4) {
        int a = bi < 4 ? 0 : (bi < 7 ? 1 : (bi < 9 ? 2 : 3));
        int b = a + (bi - (a == 0 ? 0 : (a == 1 ? 4 : (a == 2 ? 7 : 9))));
        R acc[6][6];
#pragma unroll
        for (int i = 0; i < 6; i++)
#pragma unroll
            for (int j = 0; j < 6; j++) acc[i][j] = 0;
        for (int rho = 0; rho < NR; rho++) {
            const R *rr = rows + rho * ND;
            R ra[6], rb[6];
#pragma unroll
            for (int i = 0; i < 6; i++) {
                ra[i] = rr[6 * a + i];
                rb[i] = rr[6 * b + i];
            }
#pragma unroll
            for (int i = 0; i < 6; i++)
#pragma unroll
                for (int j = 0; j < 6; j++) acc[i][j] += ra[i] * rb[j];
        }
        store_block<R>(out + ub(a, b, 4) * 36, acc, false);
    }
}

// Shared memory of one block of the element kernels (per-element Gram rows).
size_t t3_smem(int precision, bool avgk, int epb)
{
    const int nr = avgk ? T3Rows<true>::N : T3Rows<false>::N;
    return (precision == FS_FP64 ? 8 : 4) * (size_t)epb * (nr * 18 + 1);
}
size_t q4_smem(int precision, int epb) { return (precision == FS_FP64 ? 8 : 4) * (size_t)epb * (36 * 24 + 1); }

template <class R, bool COMP, bool AVGK, int EPB>
static int run_t3_epb(fs_ctx *c, R *ke)
{
    const size_t smem = t3_smem(sizeof(R) == 8 ? FS_FP64 : FS_MIXED, AVGK, EPB);
    auto kern = k_t3_elements<R, COMP, AVGK, EPB>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(c->mesh.nelem, EPB), EPB, smem, c->stream>>>(c->mesh, c->mc, ke, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

template <class R, bool COMP, bool AVGK>
static int run_t3(fs_ctx *c, R *ke)
{
    int epb = c->tune.elem_epb;
    if (epb <= 0) epb = (sizeof(R) == 8 && AVGK) ? 64 : 128;
    if (epb == 32) return run_t3_epb<R, COMP, AVGK, 32>(c, ke);
    if (epb == 64 || (sizeof(R) == 8 && AVGK)) return run_t3_epb<R, COMP, AVGK, 64>(c, ke);
    return run_t3_epb<R, COMP, AVGK, 128>(c, ke);
}

template <class R, bool COMP, int EPB>
static int run_q4_epb(fs_ctx *c, R *ke)
{
    const size_t smem = q4_smem(sizeof(R) == 8 ? FS_FP64 : FS_MIXED, EPB);
    auto kern = k_q4_elements<R, COMP, EPB>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(c->mesh.nelem, EPB), EPB * 4, smem, c->stream>>>(c->mesh, c->mc, ke, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

template <class R, bool COMP>
static int run_q4(fs_ctx *c, R *ke)
{
    int epb = c->tune.elem_epb;
    if (epb <= 0) epb = 32;
    if (epb == 16) return run_q4_epb<R, COMP, 16>(c, ke);
    if (epb == 64 && sizeof(R) == 4) return run_q4_epb<R, COMP, 64>(c, ke);
    return run_q4_epb<R, COMP, 32>(c, ke);
}

int launch_elements(fs_ctx *c, int precision)
{
    MeshDev &m = c->mesh;
    size_t bytes = (size_t)m.nelem * n_upper_blocks(m.nen) * 36 * (precision == FS_FP64 ? 8 : 4);
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
    bool comp = (m.etype == FS_T3FFCOMP || m.etype == FS_Q4RSCOMP);
    bool avgk = c->params.transv_shear_formulation == 1;
    if (m.nen == 3) {
        if (precision == FS_FP64) {
            double *k = (double *)c->ke;
            if (comp) return avgk ? run_t3<double, true, true>(c, k) : run_t3<double, true, false>(c, k);
            return avgk ? run_t3<double, false, true>(c, k) : run_t3<double, false, false>(c, k);
        }
        float *k = (float *)c->ke;
        if (comp) return avgk ? run_t3<float, true, true>(c, k) : run_t3<float, true, false>(c, k);
        return avgk ? run_t3<float, false, true>(c, k) : run_t3<float, false, false>(c, k);
    }
    if (precision == FS_FP64) {
        double *k = (double *)c->ke;
        return comp ? run_q4<double, true>(c, k) : run_q4<double, false>(c, k);
    }
    float *k = (float *)c->ke;
    return comp ? run_q4<float, true>(c, k) : run_q4<float, false>(c, k);
}

// ---------------------------------------------------------------------------
// gather into CSR values
// ---------------------------------------------------------------------------
// One warp per node.  The node's element slabs are staged into shared memory
// with independent coalesced loads, a few pairs at a time; each lane then
// owns whole row positions j (all six rows of the node) and adds the staged
// contributions of the pairs in ascending assembly rank.  In double
// (FS_FP64) the sum is a plain double accumulation.  For float element
// matrices (FS_MIXED) the sum is carried error-free as an unevaluated pair
// of floats (TwoSum), then rounded once to double: on GB300, where a double
// add costs as much as 64 float operations, this keeps one double add per
// stored value instead of a conversion and an add per contribution, with an
// error below 2^-46 of the largest contribution.  Rows longer than
// 32 * G_COLS positions fall back to accumulating in place in double.
static const int G_MAXP = 8;

// 16-byte asynchronous global -> shared copy (bypassing registers and L1)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// exact float -> double built from the bit pattern with integer operations
// only (zeros, subnormals, normals, inf and nan), so that no conversion
// lands on the double-precision pipe
__device__ __forceinline__ double f2d_exact(float f)
{
    const uint32_t u = __float_as_uint(f);
    const uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    uint32_t ex = a >> 23, man = a & 0x7fffffu;
    uint32_t dexp;
    if (ex == 0xffu) {
        dexp = 0x7ffu;                                   // inf / nan
    } else if (ex != 0u) {
        dexp = ex + (1023u - 127u);                      // normal
    } else if (man != 0u) {
        const uint32_t sh = (uint32_t)__clz((int)man) - 8u;  // subnormal: normalise
        man = (man << sh) & 0x7fffffu;
        dexp = 1023u - 126u - sh;
    } else {
        dexp = 0u;                                       // signed zero
    }
    return __hiloint2double((int)(sign | (dexp << 20) | (man >> 3)), (int)(man << 29));
}

// exact float -> double for normal numbers and zeros from the bit pattern
// (rebias the exponent, move the mantissa); other values take f2d_exact
__device__ __forceinline__ double f2d_fast(float f)
{
    const uint32_t u = __float_as_uint(f), a = u & 0x7fffffffu;
    if (a != 0u && a - 0x00800000u >= 0x7f000000u) return f2d_exact(f);  // subnormal, inf, nan
    const uint32_t h = (u & 0x80000000u) | (a != 0u ? (a >> 3) + 0x38000000u : 0u);
    return __hiloint2double((int)h, (int)(u << 29));
}

// shared memory of one warp: G_MAXP staged slabs, then the node's
// contribution entries (at most 64 pairs x 4 element nodes)
template <class R, int NEN> struct GatherSmem {
    static constexpr int PER_WARP = G_MAXP * NEN * 36 * (int)sizeof(R) + 512;
};

template <class R, int NEN, int G_COLS, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_gather(const MeshDev m, const PatternDev P, int64_t n, const R *ke, double *vals)
{
    constexpr int SLAB = NEN * 36, ND2 = 36 * (NEN * (NEN + 1) / 2);
    constexpr bool SINGLE = sizeof(R) == 4;
    constexpr int BCH = 36 * (int)sizeof(R) / 16;  // 16-byte chunks per 6x6 block
    constexpr int CH = NEN * BCH;                   // 16-byte chunks per slab
    constexpr int CPL = (CH + 31) / 32;             // chunks per lane per pair
    extern __shared__ __align__(16) unsigned char gather_smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t r = (int64_t)blockIdx.x * WARPS + w;
    if (r >= m.nnodes) return;
    unsigned char *wsm = gather_smem + (size_t)w * GatherSmem<R, NEN>::PER_WARP;
    R *stage = reinterpret_cast<R *>(wsm);
    uint16_t *sent = reinterpret_cast<uint16_t *>(wsm + G_MAXP * SLAB * sizeof(R));
    int32_t d[6];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        d[k] = m.dof[(int64_t)k * m.nnodes + r];
        any |= (d[k] <= n);
    }
    if (!any) return;
    const int L = P.rowlen[r];
    const int64_t off = P.nbr_off[r], off6 = off * 6;
    const int64_t pb = m.pp[r], pe = m.pp[r + 1];
    if (L <= 32 * G_COLS) {
        // the node's contribution entries into shared memory
        const int ntot = (int)(pe - pb) * NEN;
        const uint16_t *ent = P.sl_ent + pb * NEN;
        for (int i = lane; i < ntot; i += 32) sent[i] = ent[i];
        // the lane's columns and the range of entries of their neighbour slot
        const int nslots = (int)(P.nbr_off[r + 1] - off);
        int kcol[G_COLS], cur[G_COLS], last[G_COLS];
        R hi[G_COLS][6], lo[G_COLS][6];
#pragma unroll
        for (int c = 0; c < G_COLS; c++) {
            const int j = lane + 32 * c;
            kcol[c] = 0;
            cur[c] = 0;
            last[c] = 0;
            if (j < L) {
                const int cs = (int)P.colsrc[off6 + j];
                const int sl = cs / 6;
                kcol[c] = cs - 6 * sl;
                cur[c] = (int)P.sl_off[off + sl];
                last[c] = sl + 1 < nslots ? (int)P.sl_off[off + sl + 1] : ntot;
            }
#pragma unroll
            for (int k = 0; k < 6; k++) {
                hi[c][k] = 0;
                lo[c][k] = 0;
            }
        }
        // lane-fixed staging chunks: chunk lane + 32 t of every slab
        int cb[CPL], cwd[CPL];
#pragma unroll
        for (int t = 0; t < CPL; t++) {
            const int ch = lane + 32 * t;
            cb[t] = ch / BCH;
            cwd[t] = ch - cb[t] * BCH;
        }
        for (int64_t p0 = pb; p0 < pe; p0 += G_MAXP) {
            const int cnt = (int)min((int64_t)G_MAXP, pe - p0);
            const int q0 = (int)(p0 - pb);
            for (int q = 0; q < cnt; q++) {
                const int32_t pel = m.pair_e[p0 + q];
                const int a = pel & 3;
                const R *base = ke + (int64_t)(pel >> 2) * ND2;
#pragma unroll
                for (int t = 0; t < CPL; t++) {
                    if (lane + 32 * t < CH) {
                        const int bb = cb[t];
                        // block (a, bb) of the element: stored as itself or as its mirror
                        const R *src = base + ub(min(a, bb), max(a, bb), NEN) * 36;
                        cp_async16(reinterpret_cast<char *>(stage + q * SLAB + bb * 36) + 16 * cwd[t],
                                   reinterpret_cast<const char *>(src) + 16 * cwd[t]);
                    }
                }
            }
            cp_async_wait_all();
            __syncwarp();
            // this batch's contributions to the lane's columns, ascending pair order
#pragma unroll
            for (int c = 0; c < G_COLS; c++) {
                while (cur[c] < last[c]) {
                    const uint32_t e = sent[cur[c]];
                    const int q = (int)(e & 63u) - q0;
                    if (q >= cnt) break;
                    const int b = (int)((e >> 6) & 3u);
                    // entry (krow, kcol) of block (a_q, b); a mirrored block is read transposed
                    const bool tr = (e >> 8) & 1u;
                    const R *src = stage + q * SLAB + b * 36 + (tr ? 6 * kcol[c] : kcol[c]);
                    const int st = tr ? 1 : 6;
#pragma unroll
                    for (int k = 0; k < 6; k++) {
                        const R v = src[st * k];
                        if (SINGLE) {
                            const R t = hi[c][k] + v;
                            const R bp = t - hi[c][k];
                            lo[c][k] += (hi[c][k] - (t - bp)) + (v - bp);
                            hi[c][k] = t;
                        } else {
                            hi[c][k] += v;
                        }
                    }
                    cur[c]++;
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (d[k] > n) continue;
            double *o = vals + P.rowptr[d[k] - 1];
#pragma unroll
            for (int c = 0; c < G_COLS; c++) {
                const int j = lane + 32 * c;
                if (j >= L) continue;
                double v;
                if (SINGLE) {
                    // hi + lo: exact in double unless their exponents are more than
                    // 29 apart, then rounded once
                    v = f2d_fast((float)hi[c][k]);
                    if (lo[c][k] != (R)0) v += f2d_fast((float)lo[c][k]);
                } else {
                    v = (double)hi[c][k];
                }
                o[j] = v;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (d[k] > n) continue;
            double *o = vals + P.rowptr[d[k] - 1];
            for (int j = lane; j < L; j += 32) o[j] = 0.0;
        }
        __syncwarp();
        for (int64_t p = pb; p < pe; p++) {
            int32_t pe_ = m.pair_e[p];
            int64_t rank = pe_ >> 2;
            int a = pe_ & 3;
            uint32_t slots = P.pair_slots[p];
            for (int idx = lane; idx < SLAB; idx += 32) {
                int b = idx / 36, rem = idx - 36 * b, krow = rem / 6, kc = rem - 6 * krow;
                const R *blk = ke + rank * (int64_t)ND2 + ub(min(a, b), max(a, b), NEN) * 36;
                const R v = b < a ? blk[kc * 6 + krow] : blk[rem];
                int s = (slots >> (8 * b)) & 0xff;
                int cp = P.colpos[off6 + s * 6 + kc];
                if (cp >= 0 && d[krow] <= n) {
                    double *o = vals + P.rowptr[d[krow] - 1] + cp;
                    *o += (double)v;
                }
            }
            __threadfence_block();
            __syncwarp();
        }
    }
}

template <class R, int NEN, int G_COLS, int W>
static int gather_launch_w(fs_ctx *c, const R *ke, double *vals)
{
    const MeshDev &m = c->mesh;
    const size_t smem = (size_t)W * GatherSmem<R, NEN>::PER_WARP;
    auto kern = k_gather<R, NEN, G_COLS, W>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(m.nnodes, W), W * 32, smem, c->stream>>>(m, c->pat, c->pat.n, ke, vals);
    return FS_OK;
}

template <class R, int NEN, int G_COLS>
static int gather_launch_c(fs_ctx *c, const R *ke, double *vals, int warps)
{
    if (warps == 4) return gather_launch_w<R, NEN, G_COLS, 4>(c, ke, vals);
    if (warps == 16) return gather_launch_w<R, NEN, G_COLS, 16>(c, ke, vals);
    return gather_launch_w<R, NEN, G_COLS, 8>(c, ke, vals);
}

template <class R, int NEN>
static int gather_launch(fs_ctx *c, const R *ke, double *vals, int warps)
{
    // per-lane columns sized to the longest row (rows beyond 128 accumulate in place)
    if (c->pat.maxlen <= 64) return gather_launch_c<R, NEN, 2>(c, ke, vals, warps);
    return gather_launch_c<R, NEN, 4>(c, ke, vals, warps);
}

template <class R>
static int run_gather(fs_ctx *c, const R *ke, double *vals, int warps)
{
    if (warps <= 0) warps = sizeof(R) == 4 ? 8 : 4;
    int st;
    if (c->mesh.nen == 3)
        st = gather_launch<R, 3>(c, ke, vals, warps);
    else if (c->mesh.nen == 2)
        st = gather_launch<R, 2>(c, ke, vals, warps);
    else
        st = gather_launch<R, 4>(c, ke, vals, warps);
    FS_TRY(st);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

int launch_gather(fs_ctx *c, int precision, double *vals)
{
    if (c->mesh.nnodes == 0) return FS_OK;
    const int w = c->tune.gather_warps;
    if (precision == FS_FP64) return run_gather<double>(c, (const double *)c->ke, vals, w);
    return run_gather<float>(c, (const float *)c->ke, vals, w);
}

// ---------------------------------------------------------------------------
// nodal normals (associategeometry!)
// ---------------------------------------------------------------------------
template <int NN>
__device__ void elem_node_normal(const MeshDev &m, int64_t rank, int a, bool comp, double nn[3])
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
        const double *cs = m.groups[m.group[rank]].csmat;
        for (int c = 0; c < 3; c++) nn[c] = jac * cs[6 + c];
    } else {
        double e[3][3];
        make_frame(J0, J1, e);
        for (int c = 0; c < 3; c++) nn[c] = jac * e[2][c];
    }
}

template <int NN>
__global__ void k_normals(const MeshDev m, bool comp, double cos_thr, double *normals, uint8_t *valid)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nnodes) return;
    double s[3] = {0, 0, 0};
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        int32_t v = m.pair_e[p];
        double nn[3];
        elem_node_normal<NN>(m, v >> 2, v & 3, comp, nn);
        for (int c = 0; c < 3; c++) s[c] += nn[c];
    }
    double len = sqrt(dot3(s, s));
    if (len > 0.0)
        for (int c = 0; c < 3; c++) s[c] /= len;
    bool ok = true;
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        int32_t v = m.pair_e[p];
        double nn[3];
        elem_node_normal<NN>(m, v >> 2, v & 3, comp, nn);
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

int launch_normals(fs_ctx *c)
{
    MeshDev &m = c->mesh;
    if (m.nnodes == 0) return FS_OK;
    double th = c->params.threshold_angle;
    double sn = sin(th / 180.0 * M_PI);
    double ntol = 1 - sqrt(1 - sn * sn);
    double cos_thr = 1 - ntol;
    bool comp = (m.etype == FS_T3FFCOMP || m.etype == FS_Q4RSCOMP);
    if (m.nen == 3)
        k_normals<3><<<nblk2(m.nnodes, 128), 128, 0, c->stream>>>(m, comp, cos_thr, m.normals, m.valid);
    else
        k_normals<4><<<nblk2(m.nnodes, 128), 128, 0, c->stream>>>(m, comp, cos_thr, m.normals, m.valid);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
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
    MeshDev &m = c->mesh;
    if (m.nelem == 0) return FS_OK;
    bool comp = (m.etype == FS_T3FFCOMP || m.etype == FS_Q4RSCOMP);
    bool avgk = c->params.transv_shear_formulation == 1;
    if (m.nen == 3) {
        if (precision == FS_FP64) {
            double *k = (double *)ke;
            if (comp) return avgk ? run_t3<double, true, true>(c, k) : run_t3<double, true, false>(c, k);
            return avgk ? run_t3<double, false, true>(c, k) : run_t3<double, false, false>(c, k);
        }
        float *k = (float *)ke;
        if (comp) return avgk ? run_t3<float, true, true>(c, k) : run_t3<float, true, false>(c, k);
        return avgk ? run_t3<float, false, true>(c, k) : run_t3<float, false, false>(c, k);
    }
    if (precision == FS_FP64) {
        double *k = (double *)ke;
        return comp ? run_q4<double, true>(c, k) : run_q4<double, false>(c, k);
    }
    float *k = (float *)ke;
    return comp ? run_q4<float, true>(c, k) : run_q4<float, false>(c, k);
}

// CSR values from element matrices held in `ke`; allocates nothing.
int launch_gather_from(fs_ctx *c, int precision, const void *ke, double *vals)
{
    if (c->mesh.nnodes == 0) return FS_OK;
    const int w = c->tune.gather_warps;
    if (precision == FS_FP64) return run_gather<double>(c, (const double *)ke, vals, w);
    return run_gather<float>(c, (const float *)ke, vals, w);
}

// ---------------------------------------------------------------------------
// tile-shape autotuner
// ---------------------------------------------------------------------------
// Candidates: elements per block of the element kernel (T3: 32, 64, 128;
// Q4: 16, 32, 64, as far as their shared memory fits in 227 KB) and warps
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
std::map<TuneKey, std::pair<int, int>> g_tune;
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
    if (c->tune.mode == 0 || m.nelem < TUNE_MIN_ELEMENTS) {
        c->tune.elem_epb = 0;
        c->tune.gather_warps = 0;
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
            c->tune.elem_epb = it->second.first;
            c->tune.gather_warps = it->second.second;
            c->tune.from_tuner = true;
            return FS_OK;
        }
    }
    const bool t3 = m.nen == 3;
    const int ecand[3] = {t3 ? 32 : 16, t3 ? 64 : 32, t3 ? 128 : 64};
    int best_e = 0;
    float best_ms = 1e30f;
    for (int epb : ecand) {
        const size_t smem = t3 ? t3_smem(precision, avgk, epb) : q4_smem(precision, epb);
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
    int best_w = 0;
    best_ms = 1e30f;
    for (int w : {4, 8, 16}) {
        c->tune.gather_warps = w;
        float ms = 0.f;
        FS_TRY(time_best(c, run_gather_once, precision, &ms));
        if (ms < best_ms) {
            best_ms = ms;
            best_w = w;
        }
    }
    c->tune.gather_warps = best_w;
    c->tune.from_tuner = true;
    if (c->tune.mode == 2) c->tune.mode = 1;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = {best_e, best_w};
    return FS_OK;
}

}  // namespace fs

// CSR value gather (see the description below).
#include <type_traits>

#include "fs_elem_common.cuh"

namespace fs {

// ---------------------------------------------------------------------------
// gather into CSR values
// ---------------------------------------------------------------------------
// One warp per node.  The node's element slabs are staged into shared memory
// with independent coalesced loads, a few pairs at a time; each lane then
// owns whole row positions j (all six rows of the node) and adds the staged
// contributions of the pairs in ascending assembly rank.  In double
// (FS_FP64) the sum is a plain double accumulation.  For float element
// matrices (FS_MIXED) the sum is carried as an unevaluated pair of floats
// (TwoSum into the high part, its errors summed in the low part), then
// rounded once to double: on GB300, where a double add costs as much as 64
// float operations, this keeps one double add per stored value instead of a
// conversion and an add per contribution, with an error below 2^-46 of the
// largest contribution.  Float-pair element matrices
// (FS_MIXED_COMP) are summed into a float triple, which loses only its tail's
// float rounding (at most 8 n^2 (n + 1) 2^-72 of the n contributions'
// magnitudes; on ill-conditioned sums of up to 12 contributions below 2^-73
// of the largest), and rounded to double with two adds.  Rows longer than
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

// The six sums (rows k = 0..5 of the node) of one of a lane's row positions.
// set() takes the first contribution, add() the next ones (src[st k]: the
// six entries of a stored block's column or, transposed, its row), value(k)
// the sum rounded to double.  Double entries: double addition.  Float
// entries: an unevaluated float pair, the high sum's error added to the low
// part (TwoSum), the low part's rounding left.  Float-pair entries
// (FS_MIXED_COMP): an unevaluated float triple, the stored high half added
// to the high part and the stored low half and the high sum's error to the
// low part by TwoSum, the low part's errors going to the tail, so that what
// is lost is the tail's rounding (about 2^-72 of the contributions) instead
// of the low part's (2^-48); rows k and k + 1 in one packed register pair.
template <class R> struct ColSum;
template <> struct ColSum<double> {
    double v[6];
    __device__ __forceinline__ void set(const double *src, int st)
    {
#pragma unroll
        for (int k = 0; k < 6; k++) v[k] = src[st * k];
    }
    __device__ __forceinline__ void add(const double *src, int st)
    {
#pragma unroll
        for (int k = 0; k < 6; k++) v[k] += src[st * k];
    }
    __device__ __forceinline__ double value(int k) const { return v[k]; }
};
__device__ __forceinline__ float two_sum_err(float &s, float v)
{
    const float t = s + v;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (v - bp);
    s = t;
    return e;
}
template <> struct ColSum<float> {
    float hi[6], lo[6];
    __device__ __forceinline__ void set(const float *src, int st)
    {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            hi[k] = src[st * k];
            lo[k] = 0.f;
        }
    }
    __device__ __forceinline__ void add(const float *src, int st)
    {
#pragma unroll
        for (int k = 0; k < 6; k++) lo[k] += two_sum_err(hi[k], src[st * k]);
    }
    // hi + lo: exact in double unless their exponents are more than 29
    // apart, then rounded once
    __device__ __forceinline__ double value(int k) const
    {
        double v = f2d_fast(hi[k]);
        if (lo[k] != 0.f) v += f2d_fast(lo[k]);
        return v;
    }
};
template <> struct ColSum<float2> {
    f32x2 hi[3], lo[3], tl[3];
    // a stored float pair is normalised (|lo| <= ulp(hi)/2): taken as is
    __device__ __forceinline__ void set(const float2 *src, int st)
    {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float2 u = src[st * 2 * q], w = src[st * (2 * q + 1)];
            hi[q] = x2_pack(u.x, w.x);
            lo[q] = x2_pack(u.y, w.y);
            tl[q] = 0ull;
        }
    }
    __device__ __forceinline__ void add(const float2 *src, int st)
    {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float2 u = src[st * 2 * q], w = src[st * (2 * q + 1)];
            x2_triple_add(hi[q], lo[q], tl[q], x2_pack(u.x, w.x), x2_pack(u.y, w.y));
        }
    }
    // hi + (lo + tl): lo + tl exact in double, then one rounding of the
    // whole to double (2^-53 of the value).  Ending in a float rounding of
    // the low parts instead (one double add, 2^-48 of the value) raised the
    // 20-eigenvalue error of the 256 x 256 layered plate from 1.1e-7 to
    // 2.8e-7: the soft modes amplify per-entry errors about 1e8-fold.
    __device__ __forceinline__ double value(int k) const
    {
        float h0, h1, l0, l1, t0, t1;
        x2_unpack(hi[k >> 1], h0, h1);
        x2_unpack(lo[k >> 1], l0, l1);
        x2_unpack(tl[k >> 1], t0, t1);
        return triple_value((k & 1) ? h1 : h0, (k & 1) ? l1 : l0, (k & 1) ? t1 : t0);
    }
};
__device__ __forceinline__ double entry_value(float v) { return (double)v; }
__device__ __forceinline__ double entry_value(double v) { return v; }
__device__ __forceinline__ double entry_value(float2 v) { return (double)v.x + (double)v.y; }

// shared memory of one warp: G_MAXP staged slabs, then the node's
// contribution entries (at most 64 pairs x 4 element nodes)
template <class R, int NEN> struct GatherSmem {
    static constexpr int PER_WARP = G_MAXP * NEN * 36 * (int)sizeof(R) + 512;
};

// resident blocks asked of the compiler: 32 warps per SM where the kernel fits
// 64 registers without spilling (float entries of three-node elements), 28
// for other float entries, 24 (at most 80 registers) for double entries and
// 20 (102) for float pairs; the one-column variant 40 (48 registers) for
// float entries of three-node elements, 36 (56) for the other float and the
// double entries, 28 (72) for float pairs (whose float triples take 18
// registers; shared memory holds the 4-warp blocks to 28 warps anyway); no
// bound for the four-column variant of long rows
template <class R, int NEN, int G_COLS, int WARPS, int G_OUT> struct GatherMinBlocks {
    static constexpr bool pair = sizeof(R) == 8 && !std::is_same<R, double>::value;
    static constexpr int warps =
        G_COLS > 2 ? 1
                   : (G_OUT == 1 ? (pair ? 28 : (sizeof(R) == 4 && NEN == 3 ? 40 : 36))
                                 : (pair ? 20 : (sizeof(R) == 4 ? (NEN == 3 ? 32 : 28) : 24)));
    static constexpr int value = warps / WARPS > 0 ? warps / WARPS : 1;
};

// G_COLS: row positions per lane (32 G_COLS: the longest row of the register
// path); G_OUT: positions a lane sums (G_OUT = 1 when every node sums at most
// 32 positions with the pairs summed once)
template <class R, int NEN, int G_COLS, int WARPS, int G_OUT>
__global__ void __launch_bounds__(WARPS * 32, (GatherMinBlocks<R, NEN, G_COLS, WARPS, G_OUT>::value))
    k_gather(const MeshDev m, const PatternDev P, int64_t n, const R *ke, double *vals, bool once)
{
    constexpr int SLAB = NEN * 36, ND2 = 36 * (NEN * (NEN + 1) / 2);
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
    // the node's scalar data: all independent loads issued together
    int32_t d[6];
#pragma unroll
    for (int k = 0; k < 6; k++) d[k] = m.dof[(int64_t)k * m.nnodes + r];
    const int L = P.rowlen[r];
    const int64_t off = P.nbr_off[r], off_next = P.nbr_off[r + 1], off6 = off * 6;
    const int64_t pb = m.pp[r], pe = m.pp[r + 1];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 6; k++) any |= (d[k] <= n);
    if (!any) return;
    if (L <= 32 * G_COLS) {
        // second round of loads, all depending only on the first: lane k < 6
        // the row pointer of dof k, lane s the first entry of neighbour slot s
        // and its pair flags, lane q the pair q of the first batch, every lane
        // its columns
        int64_t rp_l = -1;  // -1: the dof has no row
        {
            int dl = d[0];
#pragma unroll
            for (int k = 1; k < 6; k++) dl = lane == k ? d[k] : dl;
            if (lane < 6 && dl <= n) rp_l = P.rowptr[dl - 1];
        }
        const int ntot = (int)(pe - pb) * NEN;
        const int nslots = (int)(off_next - off);
        const bool slot_shfl = nslots < 32;  // slot starts exchanged by shuffles
        // node-block pairs summed once: this node qualifies (register path,
        // slot data in lanes); a lower neighbour that qualifies writes the
        // pair's values into this node's rows, an upper one that qualifies
        // gets them from this node
        const bool sym = once && slot_shfl && P.sym;
        constexpr uint32_t QBIT = G_COLS == 2 ? 4u : 8u;
        int sl_l = 0, nb_l = 0;
        uint32_t mf_l = 0;  // the slot's mirror index << 4 | flags
        if (slot_shfl && lane <= nslots) sl_l = lane < nslots ? (int)P.sl_off[off + lane] : ntot;
        if (sym && lane < nslots) {
            mf_l = (uint32_t)P.sl_mir[off + lane];
            nb_l = P.nbr[off + lane];
        }
        int32_t pel_l = lane < G_MAXP && pb + lane < pe ? m.pair_e[pb + lane] : 0;
        int cs_l[G_COLS];
#pragma unroll
        for (int c = 0; c < G_COLS; c++) {
            const int j = lane + 32 * c;
            cs_l[c] = j < L ? (int)P.colsrc[off6 + j] : 0;
        }
        // the node's contribution entries into shared memory; when all the
        // node's pairs fit one staging batch (the usual case) each entry is
        // stored decoded: its slab offset q SLAB + b 36, mirrored flag in bit 15
        const bool one_batch = pe - pb <= G_MAXP;
        const uint16_t *ent = P.sl_ent + pb * NEN;
        for (int i = lane; i < ntot; i += 32) {
            const uint32_t e = ent[i];
            sent[i] = one_batch ? (uint16_t)((e & 63u) * SLAB + ((e >> 6) & 3u) * 36 | ((e >> 8) & 1u) << 15)
                                : (uint16_t)e;
        }
        // the row positions this warp sums (all of them, or all but those of
        // lower qualifying neighbours), packed densely over the lanes through
        // the staging area: position | colsrc << 8
        int jcol[G_OUT], csc[G_OUT];
        if (sym) {
            uint32_t *pmap = reinterpret_cast<uint32_t *>(stage);
            int base = 0;
#pragma unroll
            for (int c = 0; c < G_COLS; c++) {
                const int j = lane + 32 * c;
                const uint32_t f = __shfl_sync(0xffffffffu, mf_l, cs_l[c] / 6);
                const bool mine = j < L && !((f & 1u) && (f & QBIT));
                const uint32_t mask = __ballot_sync(0xffffffffu, mine);
                if (mine) pmap[base + __popc(mask & ((1u << lane) - 1u))] = (uint32_t)j | (uint32_t)cs_l[c] << 8;
                base += __popc(mask);
            }
            __syncwarp();
#pragma unroll
            for (int c = 0; c < G_OUT; c++) {
                const int i = lane + 32 * c;
                const uint32_t v = i < base ? pmap[i] : 0u;
                jcol[c] = i < base ? (int)(v & 255u) : -1;
                csc[c] = (int)(v >> 8);
            }
            __syncwarp();
        } else {
#pragma unroll
            for (int c = 0; c < G_OUT; c++) {
                const int j = lane + 32 * c;
                jcol[c] = j < L ? j : -1;
                csc[c] = cs_l[c];
            }
        }
        // the lane's columns and the range of entries of their neighbour slot
        int kcol[G_OUT], cur[G_OUT], beg[G_OUT], last[G_OUT], slc[G_OUT];
        ColSum<R> sum[G_OUT];
#pragma unroll
        for (int c = 0; c < G_OUT; c++) {
            const int sl = csc[c] / 6;
            slc[c] = sl;
            kcol[c] = csc[c] - 6 * sl;
            int b0, b1;
            if (slot_shfl) {
                b0 = __shfl_sync(0xffffffffu, sl_l, sl);
                b1 = __shfl_sync(0xffffffffu, sl_l, sl + 1);
            } else {
                b0 = (int)P.sl_off[off + sl];
                b1 = sl + 1 < nslots ? (int)P.sl_off[off + sl + 1] : ntot;
            }
            cur[c] = jcol[c] >= 0 ? b0 : 0;
            last[c] = jcol[c] >= 0 ? b1 : 0;
            beg[c] = cur[c];
            // sum[c]: set by the first contribution (every row position has one)
        }
        // lane-fixed staging chunks: chunk lane + 32 t of every slab
        int cb[CPL], cwd[CPL];
#pragma unroll
        for (int t = 0; t < CPL; t++) {
            const int ch = lane + 32 * t;
            cb[t] = ch / BCH;
            cwd[t] = ch - cb[t] * BCH;
        }
        if (one_batch) {
            // all pairs of the node in one batch (the usual case): every
            // contribution is staged, each sum runs over its whole list
            const int cnt = (int)(pe - pb);
            for (int q = 0; q < cnt; q++) {
                const int32_t pel = __shfl_sync(0xffffffffu, pel_l, q);
                const int a = pel & 3;
                const R *base = ke + (int64_t)(pel >> 2) * ND2;
#pragma unroll
                for (int t = 0; t < CPL; t++) {
                    if (lane + 32 * t < CH) {
                        const int bb = cb[t];
                        const R *src = base + ub(min(a, bb), max(a, bb), NEN) * 36;
                        cp_async16(reinterpret_cast<char *>(stage + q * SLAB + bb * 36) + 16 * cwd[t],
                                   reinterpret_cast<const char *>(src) + 16 * cwd[t]);
                    }
                }
            }
            cp_async_wait_all();
            __syncwarp();
#pragma unroll
            for (int c = 0; c < G_OUT; c++) {
                int e = cur[c];
                const int e1 = last[c];
                if (e < e1) {
                    // decoded entry: slab offset, mirrored blocks read transposed
                    const int kc = kcol[c], kc6 = 6 * kcol[c];
                    uint32_t d = sent[e];
                    bool tr = d >> 15;
                    const R *src = stage + (d & 0x7fffu) + (tr ? kc6 : kc);
                    int st = tr ? 1 : 6;
                    sum[c].set(src, st);
                    for (e++; e < e1; e++) {
                        d = sent[e];
                        tr = d >> 15;
                        src = stage + (d & 0x7fffu) + (tr ? kc6 : kc);
                        st = tr ? 1 : 6;
                        sum[c].add(src, st);
                    }
                }
            }
        } else
        for (int64_t p0 = pb; p0 < pe; p0 += G_MAXP) {
            const int cnt = (int)min((int64_t)G_MAXP, pe - p0);
            const int q0 = (int)(p0 - pb);
            if (p0 != pb) pel_l = lane < cnt ? m.pair_e[p0 + lane] : 0;
            for (int q = 0; q < cnt; q++) {
                const int32_t pel = __shfl_sync(0xffffffffu, pel_l, q);
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
            for (int c = 0; c < G_OUT; c++) {
                // the value's first contribution initialises the sum
                if (cur[c] == beg[c] && cur[c] < last[c]) {
                    const uint32_t e = sent[cur[c]];
                    const int q = (int)(e & 63u) - q0;
                    if (q < cnt) {
                        const int b = (int)((e >> 6) & 3u);
                        const bool tr = (e >> 8) & 1u;
                        const R *src = stage + q * SLAB + b * 36 + (tr ? 6 * kcol[c] : kcol[c]);
                        const int st = tr ? 1 : 6;
                        sum[c].set(src, st);
                        cur[c]++;
                    }
                }
                while (cur[c] < last[c]) {
                    const uint32_t e = sent[cur[c]];
                    const int q = (int)(e & 63u) - q0;
                    if (q >= cnt) break;
                    const int b = (int)((e >> 6) & 3u);
                    // entry (krow, kcol) of block (a_q, b); a mirrored block is read transposed
                    const bool tr = (e >> 8) & 1u;
                    const R *src = stage + q * SLAB + b * 36 + (tr ? 6 * kcol[c] : kcol[c]);
                    const int st = tr ? 1 : 6;
                    sum[c].add(src, st);
                    cur[c]++;
                }
            }
            __syncwarp();
        }
        // write-out, column by column; a column of an upper qualifying
        // neighbour s puts its six values also into row (s, kcol), at the
        // positions of this node's dofs in s's rows
#pragma unroll
        for (int c = 0; c < G_OUT; c++) {
            const uint32_t f = __shfl_sync(0xffffffffu, mf_l, slc[c]);
            const int snode = __shfl_sync(0xffffffffu, nb_l, slc[c]);
            const bool tw = jcol[c] >= 0 && (f & 2u) && (f & QBIT);
            int64_t trow = 0;
            uint32_t tcp[3] = {0u, 0u, 0u};
            if (tw) {
                const int32_t dc = m.dof[(int64_t)kcol[c] * m.nnodes + snode];
                trow = P.rowptr[dc - 1];
                const uint32_t *cp = reinterpret_cast<const uint32_t *>(P.colpos + 6 * (int64_t)(f >> 4));
                tcp[0] = cp[0];
                tcp[1] = cp[1];
                tcp[2] = cp[2];
            }
#pragma unroll
            for (int k = 0; k < 6; k++) {
                const int64_t rpk = __shfl_sync(0xffffffffu, rp_l, k);
                if (rpk < 0 || jcol[c] < 0) continue;
                const double v = sum[c].value(k);
                vals[rpk + jcol[c]] = v;
                if (tw) vals[trow + (int16_t)(tcp[k >> 1] >> (16 * (k & 1)))] = v;
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
                int dk = d[0];  // d[krow] without a local-memory copy of d
#pragma unroll
                for (int k = 1; k < 6; k++) dk = krow == k ? d[k] : dk;
                if (cp >= 0 && dk <= n) {
                    double *o = vals + P.rowptr[dk - 1] + cp;
                    *o += entry_value(v);
                }
            }
            __threadfence_block();
            __syncwarp();
        }
    }
}

template <class R, int NEN, int G_COLS, int W, int G_OUT>
static int gather_launch_w(fs_ctx *c, const R *ke, double *vals)
{
    const MeshDev &m = c->mesh;
    const size_t smem = (size_t)W * GatherSmem<R, NEN>::PER_WARP;
    auto kern = k_gather<R, NEN, G_COLS, W, G_OUT>;
    FS_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nblk2(m.nnodes, W), W * 32, smem, c->stream>>>(m, c->pat, c->pat.n, ke, vals, c->tune.gather_once != 0);
    return FS_OK;
}

template <class R, int NEN, int G_COLS, int G_OUT>
static int gather_launch_c(fs_ctx *c, const R *ke, double *vals, int warps)
{
    if (warps == 4) return gather_launch_w<R, NEN, G_COLS, 4, G_OUT>(c, ke, vals);
    if (warps == 16) return gather_launch_w<R, NEN, G_COLS, 16, G_OUT>(c, ke, vals);
    return gather_launch_w<R, NEN, G_COLS, 8, G_OUT>(c, ke, vals);
}

template <class R, int NEN>
static int gather_launch(fs_ctx *c, const R *ke, double *vals, int warps)
{
    // per-lane columns sized to the longest row (rows beyond 128 accumulate in place)
    if (c->pat.maxlen <= 64) {
        // one summed position per lane when the pairs are summed once and no
        // node sums more than 32 positions
        if (c->tune.gather_once != 0 && c->pat.sym && c->pat.maxlc <= 32)
            return gather_launch_c<R, NEN, 2, 1>(c, ke, vals, warps);
        return gather_launch_c<R, NEN, 2, 2>(c, ke, vals, warps);
    }
    return gather_launch_c<R, NEN, 4, 4>(c, ke, vals, warps);
}

size_t gather_smem_bytes(int precision, int nen, int warps)
{
    return (size_t)warps * ((size_t)G_MAXP * nen * 36 * entry_bytes(precision) + 512);
}

template <class R>
static int run_gather(fs_ctx *c, const R *ke, double *vals, int warps)
{
    if (warps <= 0) warps = sizeof(R) == 4 ? 8 : 4;  // double and float-pair entries: 4
    const int prec = sizeof(R) == 4 ? FS_MIXED : FS_FP64;  // float pairs have double's entry size
    while (warps > 4 && gather_smem_bytes(prec, c->mesh.nen, warps) > 227 * 1024) warps /= 2;
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
    if (precision == FS_MIXED_COMP) return run_gather<float2>(c, (const float2 *)c->ke, vals, w);
    return run_gather<float>(c, (const float *)c->ke, vals, w);
}

// CSR values from element matrices held in `ke`; allocates nothing.
int launch_gather_from(fs_ctx *c, int precision, const void *ke, double *vals)
{
    if (c->mesh.nnodes == 0) return FS_OK;
    const int w = c->tune.gather_warps;
    if (precision == FS_FP64) return run_gather<double>(c, (const double *)ke, vals, w);
    if (precision == FS_MIXED_COMP) return run_gather<float2>(c, (const float2 *)ke, vals, w);
    return run_gather<float>(c, (const float *)ke, vals, w);
}

}  // namespace fs

// Device helpers shared by the element kernels (T3 and Q4 translation units)
// and the numeric phase: element input loading and the stores of the upper
// node blocks of an element matrix.
#pragma once

#include "fs_internal.cuh"

namespace fs {

static inline unsigned nblk2(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

template <int NN>
__device__ __forceinline__ void load_elem(const MeshDev &m, int64_t r, ElemIn<NN> &in)
{
    for (int a = 0; a < NN; a++) {
        int node = m.conn[r * NN + a];
        for (int c = 0; c < 3; c++) {
            in.X[a][c] = m.xyz[(int64_t)c * m.nnodes + node];
            in.nrm[a][c] = m.normals[(int64_t)c * m.nnodes + node];
            in.nrmf[a][c] = m.normals_f[(int64_t)c * m.nnodes + node];
        }
        in.valid[a] = m.valid[node] != 0;
    }
    in.t = m.thick ? m.thick[r] : 0.0;
    in.group = m.group ? m.group[r] : 0;
}

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

// One step of an error-free dot product (Ogita, Rump and Oishi's Dot2):
// the product a*b is split exactly with an FMA and added to (s, c) by
// TwoSum.  The _rn intrinsics are never contracted or reassociated.
__device__ __forceinline__ void dot2_step(float &s, float &c, float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float pl = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    c = __fadd_rn(c, __fadd_rn(e, pl));
    s = t;
}

// 36 entries (s + c) of a compensated block as float pairs (hi, lo), hi the
// rounded sum and lo its error (Fast2Sum), with 16-byte stores
__device__ __forceinline__ void store_block_pair(float2 *o, const float (&s)[6][6], const float (&c)[6][6])
{
    float4 *o4 = reinterpret_cast<float4 *>(o);
#pragma unroll
    for (int q = 0; q < 18; q++) {
        float h[2], l[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int i = (2 * q + u) / 6, j = (2 * q + u) % 6;
            h[u] = __fadd_rn(s[i][j], c[i][j]);
            l[u] = __fsub_rn(c[i][j], __fsub_rn(h[u], s[i][j]));
        }
        o4[q] = make_float4(h[0], l[0], h[1], l[1]);
    }
}

// Accumulator of one 6x6 node block of K = sum_rho row_rho row_rho^T: plain
// in the row type, or (float rows into float pairs) error-free by Dot2.
template <class R, bool PAIR> struct BlockAcc {
    R v[6][6];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int i = 0; i < 6; i++)
#pragma unroll
            for (int j = 0; j < 6; j++) v[i][j] = 0;
    }
    __device__ __forceinline__ void add(int i, int j, R x, R y) { v[i][j] += x * y; }
    template <class S> __device__ __forceinline__ void store(S *o) { store_block<R>(reinterpret_cast<R *>(o), v, false); }
};
template <> struct BlockAcc<float, true> {
    float s[6][6], c[6][6];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int i = 0; i < 6; i++)
#pragma unroll
            for (int j = 0; j < 6; j++) s[i][j] = c[i][j] = 0.f;
    }
    __device__ __forceinline__ void add(int i, int j, float x, float y) { dot2_step(s[i][j], c[i][j], x, y); }
    template <class S> __device__ __forceinline__ void store(S *o) { store_block_pair(reinterpret_cast<float2 *>(o), s, c); }
};

// acc += sum over rows [r0, r1) of row[6a + i] row[6b + j] for i in
// [I0, I1), j in [J0, J1): the sub-blocks a row can reach
template <int I0, int I1, int J0, int J1, class R, class Acc>
__device__ __forceinline__ void gram_rows(Acc &acc, const R *rows, int ND, int r0, int r1, int a, int b)
{
    for (int rho = r0; rho < r1; rho++) {
        const R *rr = rows + rho * ND;
        R ra[6], rb[6];
#pragma unroll
        for (int i = I0; i < I1; i++) ra[i] = rr[6 * a + i];
#pragma unroll
        for (int j = J0; j < J1; j++) rb[j] = rr[6 * b + j];
#pragma unroll
        for (int i = I0; i < I1; i++)
#pragma unroll
            for (int j = J0; j < J1; j++) acc.add(i, j, ra[i], rb[j]);
    }
}

// acc += sum over rows [r0, r1) (stride RS from base) of row[NSTR a + i - IOFF]
// row[NSTR b + j - IOFF] for i in [I0, I1), j in [J0, J1): the same products
// as gram_rows on a compact row layout (rows holding a subset of the dofs)
template <int I0, int I1, int J0, int J1, int RS, int NSTR, int IOFF, class R, class Acc>
__device__ __forceinline__ void gram_rows_c(Acc &acc, const R *base, int r0, int r1, int a, int b)
{
    for (int rho = r0; rho < r1; rho++) {
        const R *rr = base + rho * RS;
        R ra[6], rb[6];
#pragma unroll
        for (int i = I0; i < I1; i++) ra[i] = rr[NSTR * a + i - IOFF];
#pragma unroll
        for (int j = J0; j < J1; j++) rb[j] = rr[NSTR * b + j - IOFF];
#pragma unroll
        for (int i = I0; i < I1; i++)
#pragma unroll
            for (int j = J0; j < J1; j++) acc.add(i, j, ra[i], rb[j]);
    }
}

// Upper node blocks of a homogeneous element from its rows in the
// CompactRows<NN, NS> layout: the products and their order are those of the
// SPARSE path of write_blocks, so the blocks are bitwise the same.
template <class R, class S, int NN, int NS>
__device__ __forceinline__ void write_blocks_compact(const R *rows, S *out)
{
    typedef CompactRows<NN, NS> L;
    constexpr bool PAIR = sizeof(S) == 8 && sizeof(R) == 4;
    for (int a = 0; a < NN; a++)
        for (int b = a; b < NN; b++) {
            BlockAcc<R, PAIR> acc;
            acc.zero();
            gram_rows_c<0, 3, 0, 3, L::MS, 3, 0>(acc, rows, 0, 3, a, b);
            gram_rows_c<0, 6, 0, 6, L::BSS, 6, 0>(acc, rows + L::BS, 0, 3 + NS, a, b);
            if (a == b) gram_rows_c<3, 6, 3, 6, 3, 0, 3>(acc, rows + L::DR + 3 * a, 0, 1, a, b);
            acc.store(out + ub(a, b, NN) * 36);
        }
}

// Upper node blocks of K = sum_rho row_rho row_rho^T.  Storage S: the row
// type R itself, or float2 pairs for float rows accumulated error-free
// (FS_MIXED_COMP).  SPARSE (homogeneous shells): rows 0..2 are membrane rows
// (nodal translations only) and the last NN rows drilling rows (the
// rotations of one node each); their structurally zero products are
// skipped, in the same row order, so the sums are those of the dense loop.
template <class R, class S, int NN, bool SPARSE>
__device__ __forceinline__ void write_blocks(const R *rows, int nrows, S *out)
{
    constexpr bool PAIR = sizeof(S) == 8 && sizeof(R) == 4;
    const int ND = 6 * NN;
    for (int a = 0; a < NN; a++)
        for (int b = a; b < NN; b++) {
            BlockAcc<R, PAIR> acc;
            acc.zero();
            if (SPARSE) {
                gram_rows<0, 3, 0, 3>(acc, rows, ND, 0, 3, a, b);
                gram_rows<0, 6, 0, 6>(acc, rows, ND, 3, nrows - NN, a, b);
                if (a == b) gram_rows<3, 6, 3, 6>(acc, rows, ND, nrows - NN + a, nrows - NN + a + 1, a, b);
            } else {
                gram_rows<0, 6, 0, 6>(acc, rows, ND, 0, nrows, a, b);
            }
            acc.store(out + ub(a, b, NN) * 36);
        }
}

}  // namespace fs

// Device helpers shared by the element kernels (T3 and Q4 translation units)
// and the numeric phase: element input loading and the stores of the upper
// node blocks of an element matrix.
#pragma once

#include "fs_comp_sum.cuh"
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

// NI rows of a 6x6 block (6 NI contiguous values from a 16-byte boundary for
// whole blocks, an 8-byte one for the half-blocks of float values): 16-byte
// stores, or 8-byte ones for float half-blocks
template <class R, int NI>
__device__ __forceinline__ void store_rows(R *o, const R (&acc)[NI][6])
{
    if (sizeof(R) == 4 && NI == 6) {
        float4 *o4 = reinterpret_cast<float4 *>(o);
#pragma unroll
        for (int q = 0; q < 9; q++) {
            const int e = 4 * q;
            o4[q] = make_float4((float)acc[e / 6][e % 6], (float)acc[(e + 1) / 6][(e + 1) % 6],
                                (float)acc[(e + 2) / 6][(e + 2) % 6], (float)acc[(e + 3) / 6][(e + 3) % 6]);
        }
    } else if (sizeof(R) == 4) {
        float2 *o2 = reinterpret_cast<float2 *>(o);
#pragma unroll
        for (int q = 0; q < 3 * NI; q++) o2[q] = make_float2((float)acc[q / 3][2 * (q % 3)], (float)acc[q / 3][2 * (q % 3) + 1]);
    } else {
        double2 *o2 = reinterpret_cast<double2 *>(o);
#pragma unroll
        for (int q = 0; q < 3 * NI; q++)
            o2[q] = make_double2((double)acc[q / 3][2 * (q % 3)], (double)acc[q / 3][2 * (q % 3) + 1]);
    }
}

// One step of a compensated dot product (Ogita, Rump and Oishi's Dot2):
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

// Accumulator of NI rows (6: a whole 6x6 node block of
// K = sum_rho row_rho row_rho^T; 3: half of one) in the row type.  row()
// adds the products ra[i] rb[j] of one row for i in [I0, I1), j in
// [J0, J1) (i outer, j inner; contracted to FMAs); DIAG (a diagonal block,
// ra = rb): only j >= i, store() mirroring the rest.  Products commute and
// fma(x, y, z) = fma(y, x, z), so the mirrored entries are bitwise those the
// full loop computes.
template <class R, bool PAIR, int NI = 6> struct BlockAcc {
    R v[NI][6];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int i = 0; i < NI; i++)
#pragma unroll
            for (int j = 0; j < 6; j++) v[i][j] = 0;
    }
    template <int I0, int I1, int J0, int J1, bool DIAG = false>
    __device__ __forceinline__ void row(const R (&ra)[6], const R (&rb)[6])
    {
#pragma unroll
        for (int i = I0; i < I1; i++)
#pragma unroll
            for (int j = J0; j < J1; j++)
                if (!DIAG || j >= i) v[i][j] += ra[i] * rb[j];
    }
    template <bool DIAG = false, class S> __device__ __forceinline__ void store(S *o)
    {
        if (DIAG) {
#pragma unroll
            for (int i = 1; i < NI; i++)
#pragma unroll
                for (int j = 0; j < i; j++) v[i][j] = v[j][i];
        }
        store_rows<R, NI>(reinterpret_cast<R *>(o), v);
    }
};

// Float rows into float pairs (FS_MIXED_COMP): the three-level compensated
// sums, entries (i, 2q) and (i, 2q + 1) in one packed register pair.  A row
// reaching only one entry of a pair adds a zero product to the other, which
// leaves its sums unchanged; DIAG: only the pairs holding an entry j >= i.
// store() writes s + (c + d) as (hi, lo) float pairs: c + d rounded (below
// the pair's last bit), then Fast2Sum; DIAG mirrors the entries j < i.
// LEVELS 2: Dot2 on entry pairs (s, c; what is lost is c's rounding, about
// 2^-48 of the summed terms per term summed), for elements with few rows per
// entry.
template <int NI, int LEVELS = 3> struct PairAcc {
    f32x2 s[NI][3], c[NI][3], d[NI][3];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int i = 0; i < NI; i++)
#pragma unroll
            for (int q = 0; q < 3; q++) s[i][q] = c[i][q] = d[i][q] = 0ull;
    }
    template <int I0, int I1, int J0, int J1, bool DIAG = false>
    __device__ __forceinline__ void row(const float (&ra)[6], const float (&rb)[6])
    {
        constexpr int Q0 = J0 / 2, Q1 = (J1 + 1) / 2;
        f32x2 b2[3];
#pragma unroll
        for (int q = Q0; q < Q1; q++)
            b2[q] = x2_pack(2 * q >= J0 ? rb[2 * q] : 0.f, 2 * q + 1 < J1 ? rb[2 * q + 1] : 0.f);
#pragma unroll
        for (int i = I0; i < I1; i++) {
            const f32x2 a2 = x2_pack(ra[i], ra[i]), na2 = x2_pack(-ra[i], -ra[i]);
#pragma unroll
            for (int q = Q0; q < Q1; q++)
                if (!DIAG || 2 * q + 1 >= i) {
                    if constexpr (LEVELS == 3)
                        dot3_step_x2(s[i][q], c[i][q], d[i][q], a2, na2, b2[q]);
                    else
                        dot2_step_x2(s[i][q], c[i][q], a2, na2, b2[q]);
                }
        }
    }
    template <bool DIAG = false, class S> __device__ __forceinline__ void store(S *o)
    {
        float h[NI][6], l[NI][6];
#pragma unroll
        for (int i = 0; i < NI; i++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                if (DIAG && 2 * q + 1 < i) continue;
                f32x2 hh, ll;
                x2_pair_finish<LEVELS>(s[i][q], c[i][q], d[i][q], hh, ll);
                x2_unpack(hh, h[i][2 * q], h[i][2 * q + 1]);
                x2_unpack(ll, l[i][2 * q], l[i][2 * q + 1]);
            }
        if (DIAG) {
#pragma unroll
            for (int i = 1; i < NI; i++)
#pragma unroll
                for (int j = 0; j < i; j++) {
                    h[i][j] = h[j][i];
                    l[i][j] = l[j][i];
                }
        }
        float4 *o4 = reinterpret_cast<float4 *>(o);
#pragma unroll
        for (int i = 0; i < NI; i++)
#pragma unroll
            for (int q = 0; q < 3; q++)
                o4[3 * i + q] = make_float4(h[i][2 * q], l[i][2 * q], h[i][2 * q + 1], l[i][2 * q + 1]);
    }
};
template <int NI> struct BlockAcc<float, true, NI> : PairAcc<NI, Q4_PAIR_LEVELS> {};

// acc += sum over rows [r0, r1) of row[6a + i] row[6b + j] for i in
// [I0, I1), j in [J0, J1): the sub-blocks a row can reach (DIAG: a = b, the
// upper triangle)
// The row loop of the gram helpers: unrolled, or (ROLLED) kept a loop.  The
// T3 kernel's float-pair sums run rolled: a row's body is 16 packed
// instructions per entry pair, and the unrolled loops stalled it on
// instruction fetch (21 % slower); the Q4 kernel's run faster unrolled.
template <bool ROLLED, class F>
__device__ __forceinline__ void for_rows(int r0, int r1, F body)
{
    if constexpr (ROLLED) {
#pragma unroll 1
        for (int rho = r0; rho < r1; rho++) body(rho);
    } else {
        for (int rho = r0; rho < r1; rho++) body(rho);
    }
}

template <int I0, int I1, int J0, int J1, bool DIAG = false, bool ROLLED = false, class R, class Acc>
__device__ __forceinline__ void gram_rows(Acc &acc, const R *rows, int ND, int r0, int r1, int a, int b)
{
    for_rows<ROLLED>(r0, r1, [&](int rho) {
        const R *rr = rows + rho * ND;
        R ra[6], rb[6];
#pragma unroll
        for (int i = I0; i < I1; i++) ra[i] = rr[6 * a + i];
#pragma unroll
        for (int j = J0; j < J1; j++) rb[j] = rr[6 * b + j];
        acc.template row<I0, I1, J0, J1, DIAG>(ra, rb);
    });
}

// acc += sum over rows [r0, r1) (stride RS from base) of row[NSTR a + i - IOFF]
// row[NSTR b + j - IOFF] for i in [I0, I1), j in [J0, J1): the same products
// as gram_rows on a compact row layout (rows holding a subset of the dofs)
template <int I0, int I1, int J0, int J1, int RS, int NSTR, int IOFF, bool DIAG = false, bool ROLLED = false,
          class R, class Acc>
__device__ __forceinline__ void gram_rows_c(Acc &acc, const R *base, int r0, int r1, int a, int b)
{
    for_rows<ROLLED>(r0, r1, [&](int rho) {
        const R *rr = base + rho * RS;
        R ra[6], rb[6];
#pragma unroll
        for (int i = I0; i < I1; i++) ra[i] = rr[NSTR * a + i - IOFF];
#pragma unroll
        for (int j = J0; j < J1; j++) rb[j] = rr[NSTR * b + j - IOFF];
        acc.template row<I0, I1, J0, J1, DIAG>(ra, rb);
    });
}

// Half-block forms (a three-row accumulator): rows i0 .. i0 + 2 of block
// (a, b), i0 = 0 or 3 at run time, in the stride-RS layout whose row holds
// node c's dofs k at NSTR c + k.  The products of each entry and their order
// are those of the whole-block forms.
template <int J0, int J1, int RS, int NSTR, class R, class Acc>
__device__ __forceinline__ void gram_rows_h(Acc &acc, const R *base, int r0, int r1, int a, int b, int i0)
{
    for_rows<false>(r0, r1, [&](int rho) {
        const R *rr = base + rho * RS;
        R ra[6], rb[6];
#pragma unroll
        for (int i = 0; i < 3; i++) ra[i] = rr[NSTR * a + i0 + i];
#pragma unroll
        for (int j = J0; j < J1; j++) rb[j] = rr[NSTR * b + j];
        acc.template row<0, 3, J0, J1>(ra, rb);
    });
}

// The T3 kernels' float-pair sums at T3_PAIR_LEVELS (Dot2), the Q4 kernels'
// (BlockAcc<float, true>) at Q4_PAIR_LEVELS.
template <class R, bool PAIR> struct T3Acc { typedef BlockAcc<R, PAIR> type; };
template <> struct T3Acc<float, true> { typedef PairAcc<6, T3_PAIR_LEVELS> type; };

// The upper node blocks of an NN-node element: diag(a) computes block
// (a, a) (its upper triangle), off(a, b) block (a, b) for b > a.
// Plain stores (float or double): one loop over the blocks, not unrolled,
// choosing the diagonal or the off-diagonal form (the shorter code measured
// 28 % faster for the float T3 kernel).  Float-pair stores: the diagonal
// blocks, then the off-diagonal ones (4 % faster for those).
template <int NN, bool PAIR, class D, class O>
__device__ __forceinline__ void for_upper_blocks(D diag, O off)
{
    if constexpr (PAIR) {
#pragma unroll 1
        for (int a = 0; a < NN; a++) diag(a);
#pragma unroll 1
        for (int a = 0; a < NN; a++)
#pragma unroll 1
            for (int b = a + 1; b < NN; b++) off(a, b);
    } else {
#pragma unroll 1
        for (int a = 0; a < NN; a++)
#pragma unroll 1
            for (int b = a; b < NN; b++) {
                if (a == b)
                    diag(a);
                else
                    off(a, b);
            }
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
    for_upper_blocks<NN, PAIR>(
        [&](int a) {
            typename T3Acc<R, PAIR>::type acc;
            acc.zero();
            gram_rows_c<0, 3, 0, 3, L::MS, 3, 0, true, PAIR>(acc, rows, 0, 3, a, a);
            gram_rows_c<0, 6, 0, 6, L::BSS, 6, 0, true, PAIR>(acc, rows + L::BS, 0, 3 + NS, a, a);
            gram_rows_c<3, 6, 3, 6, 3, 0, 3, true, PAIR>(acc, rows + L::DR + 3 * a, 0, 1, a, a);
            acc.template store<true>(out + ub(a, a, NN) * 36);
        },
        [&](int a, int b) {
            typename T3Acc<R, PAIR>::type acc;
            acc.zero();
            gram_rows_c<0, 3, 0, 3, L::MS, 3, 0, false, PAIR>(acc, rows, 0, 3, a, b);
            gram_rows_c<0, 6, 0, 6, L::BSS, 6, 0, false, PAIR>(acc, rows + L::BS, 0, 3 + NS, a, b);
            acc.store(out + ub(a, b, NN) * 36);
        });
}

// Upper node blocks of K = sum_rho row_rho row_rho^T.  Storage S: the row
// type R itself, or float2 pairs for float rows accumulated in compensated
// sums (FS_MIXED_COMP).  SPARSE (homogeneous shells): rows 0..2 are membrane rows
// (nodal translations only) and the last NN rows drilling rows (the
// rotations of one node each); their structurally zero products are
// skipped, in the same row order, so the sums are those of the dense loop.
template <class R, class S, int NN, bool SPARSE>
__device__ __forceinline__ void write_blocks(const R *rows, int nrows, S *out)
{
    constexpr bool PAIR = sizeof(S) == 8 && sizeof(R) == 4;
    const int ND = 6 * NN;
    for_upper_blocks<NN, PAIR>(
        [&](int a) {
            typename T3Acc<R, PAIR>::type acc;
            acc.zero();
            if (SPARSE) {
                gram_rows<0, 3, 0, 3, true, PAIR>(acc, rows, ND, 0, 3, a, a);
                gram_rows<0, 6, 0, 6, true, PAIR>(acc, rows, ND, 3, nrows - NN, a, a);
                gram_rows<3, 6, 3, 6, true, PAIR>(acc, rows, ND, nrows - NN + a, nrows - NN + a + 1, a, a);
            } else {
                gram_rows<0, 6, 0, 6, true, PAIR>(acc, rows, ND, 0, nrows, a, a);
            }
            acc.template store<true>(out + ub(a, a, NN) * 36);
        },
        [&](int a, int b) {
            typename T3Acc<R, PAIR>::type acc;
            acc.zero();
            if (SPARSE) {
                gram_rows<0, 3, 0, 3, false, PAIR>(acc, rows, ND, 0, 3, a, b);
                gram_rows<0, 6, 0, 6, false, PAIR>(acc, rows, ND, 3, nrows - NN, a, b);
            } else {
                gram_rows<0, 6, 0, 6, false, PAIR>(acc, rows, ND, 0, nrows, a, b);
            }
            acc.store(out + ub(a, b, NN) * 36);
        });
}

}  // namespace fs

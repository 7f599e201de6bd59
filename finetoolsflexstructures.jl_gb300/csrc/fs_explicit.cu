// Explicit central-difference time stepping
// (examples/shells/dynamics/homogeneous/explicit/plate_expl_examples.jl:61-94,
// _cd_loop!, with mass-proportional damping C and the external force of the
// example's force!: F(t) = g(t) Fmag, a fixed load vector times a scalar time
// function, given as its values at the step times):
//
//   U += dt V + dt^2/2 A;  F = g(t) Fmag;  E = K U;  F -= E + C (V + dt/2 A);
//   V += dt/2 A;  A = invMC F;  V += dt/2 A
//
// Two kernels per step: the displacement update, then the product K U fused
// with the force, acceleration and velocity updates of the row.  The product
// runs on 6x6 node blocks (block rows = the neighbour lists of the pattern,
// filled from the CSR matrix once at set-up, read as contiguous 144- or
// 288-byte blocks against a node-padded copy of U), or row-parallel on the CSR
// arrays when no pattern of the current mesh is at hand.  The displacement
// and velocity sums carry Kahan compensation terms so
// that a long run in double does not drift.  With FS_FP64 the restoring force
// K U is formed in double.  With FS_MIXED it is formed in float: the
// displacement kernel also writes a float copy of U and the product runs on
// float values (a double product would spend one double conversion and one
// double FMA per stored value, the scarcest pipe on GB300); the force,
// acceleration and velocity updates stay in double.  With FS_MIXED_COMP each
// value is kept as its float rounding plus the rounding's residual in bf16
// (K to about 33 bits, 6 bytes a value), the displacement copy is a float
// pair (hi, lo: U to about 48 bits), and K U is summed in compensated float
// sums (Dot2 on the float value times hi; the products with lo and with the
// residual added to the error term).  A row of K U is a small remainder of
// its terms for a smooth displacement field, so the float copy of U, the
// float sum and the float rounding of K each leave errors far above their
// own 6e-8 in it (measured in that order of size).  The step loop is
// captured once into a CUDA graph and replayed.
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "fs_elem_common.cuh"

namespace fs {

static const int CD_TPB = 256;
static const int CD_LANES = 8;  // lanes per CSR row
static const int CD_GRAPH_STEPS = 64;

// one entry of a displacement copy: double, float, or the float pair (hi, lo)
// with hi = U rounded and lo = the rest rounded
__device__ __forceinline__ void store_disp(double *p, double t) { *p = t; }
__device__ __forceinline__ void store_disp(float *p, double t) { *p = (float)t; }
__device__ __forceinline__ void store_disp(float2 *p, double t)
{
    const float h = (float)t;
    *p = make_float2(h, (float)(t - (double)h));
}

__global__ void k_cd_disp(int64_t n, double dt, double dt2_2, double *U, double *cU, const double *V,
                          const double *A, float *U32)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double y = (dt * V[i] + dt2_2 * A[i]) - cU[i];
    double u = U[i];
    double t = u + y;
    cU[i] = (t - u) - y;
    U[i] = t;
    if (U32) U32[i] = (float)t;
}

// the CSR path's displacement update writing the float-pair copy
__global__ void k_cd_disp_pair(int64_t n, double dt, double dt2_2, double *U, double *cU, const double *V,
                               const double *A, float2 *U2)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double y = (dt * V[i] + dt2_2 * A[i]) - cU[i];
    double u = U[i];
    double t = u + y;
    cU[i] = (t - u) - y;
    U[i] = t;
    store_disp(U2 + i, t);
}

// the same displacement update writing the node-padded copy read by the
// block product (entries of excluded dofs stay zero)
template <class VT>
__global__ void k_cd_disp_pad(int64_t n, double dt, double dt2_2, double *U, double *cU, const double *V,
                              const double *A, const int32_t *pad_of_dof, VT *xp)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double y = (dt * V[i] + dt2_2 * A[i]) - cU[i];
    double u = U[i];
    double t = u + y;
    cU[i] = (t - u) - y;
    U[i] = t;
    const int32_t q = pad_of_dof[i];
    if (q >= 0) store_disp(xp + q, t);
}

// six contiguous values (8-byte aligned floats, 16-byte aligned doubles)
__device__ __forceinline__ void load6(const float *p, float v[6])
{
    const float2 *q = reinterpret_cast<const float2 *>(p);
    const float2 a = q[0], b = q[1], c = q[2];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}
__device__ __forceinline__ void load6(const double *p, double v[6])
{
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = q[0], b = q[1], c = q[2];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}

// External load of step j of the current batch: the state's step index plus
// j + 1 selects g (zero past the table); null Fmag: no load.
struct CdLoad {
    const double *Fmag;
    const double *mul;
    int64_t nmul;
    const int64_t *step;
    int j;
    __device__ __forceinline__ double at(int64_t row) const
    {
        if (!Fmag) return 0.0;
        const int64_t s = *step + j + 1;
        const double g = s < nmul ? mul[s] : 0.0;
        return g * Fmag[row];
    }
};

__global__ void k_step_advance(int64_t *step, int64_t nsteps) { *step += nsteps; }

__device__ __forceinline__ void kahan_add(double &s, double &c, double incr)
{
    double y = incr - c;
    double t = s + y;
    c = (t - s) - y;
    s = t;
}

// VT: value type of K and of the displacement copy the product reads
template <class VT>
__global__ void __launch_bounds__(CD_TPB) k_cd_rows(int64_t n, const int64_t *rowptr, const int32_t *colidx,
                                                  const VT *vals, const VT *Uk, double *V, double *cV,
                                                  double *A, const double *C, const double *invMC, double dt_2,
                                                  CdLoad ld)
{
    int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / CD_LANES;
    const int sub = threadIdx.x & (CD_LANES - 1);
    const unsigned mask = 0xffffffffu;
    VT sv = 0;
    if (row < n) {
        for (int64_t k = rowptr[row] + sub; k < rowptr[row + 1]; k += CD_LANES) sv += vals[k] * Uk[colidx[k]];
    }
#pragma unroll
    for (int o = CD_LANES / 2; o > 0; o >>= 1) sv += __shfl_xor_sync(mask, sv, o);
    double s = (double)sv;
    if (row < n && sub == 0) {
        double a = A[row], v = V[row], cv = cV[row];
        double f = ld.at(row);
        f -= s + C[row] * (v + dt_2 * a);
        kahan_add(v, cv, dt_2 * a);
        a = invMC[row] * f;
        kahan_add(v, cv, dt_2 * a);
        A[row] = a;
        V[row] = v;
        cV[row] = cv;
    }
}

// K U from the 6x6 node blocks, fused with the force, acceleration and
// velocity updates: six threads per node (one per component row, five nodes
// per warp); the threads of a node read each block as 144 (float) or 288
// (double) contiguous bytes.
template <class VT>
__global__ void __launch_bounds__(CD_TPB) k_cd_bsr(int64_t nnodes, int64_t n, const int32_t *dof,
                                                 const int64_t *nbr_off, const int32_t *nbr, const VT *blk,
                                                 const VT *xp, double *V, double *cV, double *A, const double *C,
                                                 const double *invMC, double dt_2, CdLoad ld)
{
    const int t = threadIdx.x & 31;
    if (t >= 30) return;
    const int64_t r = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 5 + t / 6;
    const int i = t % 6;
    if (r >= nnodes) return;
    const int32_t d = dof[(int64_t)i * nnodes + r];
    if (d > n) return;
    VT sv = 0;
    for (int64_t b = nbr_off[r], be = nbr_off[r + 1]; b < be; b++) {
        VT kv[6], xv[6];
        load6(blk + b * 36 + i * 6, kv);
        load6(xp + (int64_t)nbr[b] * 6, xv);
#pragma unroll
        for (int j = 0; j < 6; j++) sv += kv[j] * xv[j];
    }
    const int64_t row = d - 1;
    const double s = (double)sv;
    double a = A[row], v = V[row], cv = cV[row];
    double f = ld.at(row);
    f -= s + C[row] * (v + dt_2 * a);
    kahan_add(v, cv, dt_2 * a);
    a = invMC[row] * f;
    kahan_add(v, cv, dt_2 * a);
    A[row] = a;
    V[row] = v;
    cV[row] = cv;
}

// compensated accumulation of (kv + kr) * (xh + xl) into (s, c): Dot2 on
// kv * xh, the small products kv * xl and kr * xh added to the error term
// (kr * xl is below the error of the result)
__device__ __forceinline__ void acc_pair(float &s, float &c, float kv, float kr, float2 x)
{
    dot2_step(s, c, kv, x.x);
    c = __fmaf_rn(kv, x.y, c);
    c = __fmaf_rn(kr, x.x, c);
}
// six bf16 residuals (4-byte aligned) as floats
__device__ __forceinline__ void load6_bf16(const __nv_bfloat16 *p, float v[6])
{
    const __nv_bfloat162 *q = reinterpret_cast<const __nv_bfloat162 *>(p);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float2 f = __bfloat1622float2(q[k]);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}
// (s1, c1) += (s2, c2) without losing the rounding of s1 + s2 (TwoSum)
__device__ __forceinline__ void add_pair(float &s, float &c, float s2, float c2)
{
    const float t = __fadd_rn(s, s2);
    const float z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(s2, z));
    c = __fadd_rn(__fadd_rn(c, c2), e);
    s = t;
}

// The block product of k_cd_bsr with the float-pair displacement copy and
// the compensated float sum (FS_MIXED_COMP); the rest of the step as there.
__global__ void __launch_bounds__(CD_TPB) k_cd_bsr_comp(int64_t nnodes, int64_t n, const int32_t *dof,
                                                      const int64_t *nbr_off, const int32_t *nbr, const float *blk,
                                                      const __nv_bfloat16 *res, const float2 *xp, double *V,
                                                      double *cV, double *A, const double *C, const double *invMC,
                                                      double dt_2, CdLoad ld)
{
    const int t = threadIdx.x & 31;
    if (t >= 30) return;
    const int64_t r = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 5 + t / 6;
    const int i = t % 6;
    if (r >= nnodes) return;
    const int32_t d = dof[(int64_t)i * nnodes + r];
    if (d > n) return;
    float s = 0.f, c = 0.f;
    for (int64_t b = nbr_off[r], be = nbr_off[r + 1]; b < be; b++) {
        float kv[6], kr[6];
        load6(blk + b * 36 + i * 6, kv);
        load6_bf16(res + b * 36 + i * 6, kr);
        const float4 *xq = reinterpret_cast<const float4 *>(xp + (int64_t)nbr[b] * 6);
        const float4 x01 = xq[0], x23 = xq[1], x45 = xq[2];
        acc_pair(s, c, kv[0], kr[0], make_float2(x01.x, x01.y));
        acc_pair(s, c, kv[1], kr[1], make_float2(x01.z, x01.w));
        acc_pair(s, c, kv[2], kr[2], make_float2(x23.x, x23.y));
        acc_pair(s, c, kv[3], kr[3], make_float2(x23.z, x23.w));
        acc_pair(s, c, kv[4], kr[4], make_float2(x45.x, x45.y));
        acc_pair(s, c, kv[5], kr[5], make_float2(x45.z, x45.w));
    }
    const int64_t row = d - 1;
    const double sv = (double)s + (double)c;
    double a = A[row], v = V[row], cv = cV[row];
    double f = ld.at(row);
    f -= sv + C[row] * (v + dt_2 * a);
    kahan_add(v, cv, dt_2 * a);
    a = invMC[row] * f;
    kahan_add(v, cv, dt_2 * a);
    A[row] = a;
    V[row] = v;
    cV[row] = cv;
}

// The CSR product of k_cd_rows with the float-pair displacement copy and the
// compensated float sum (FS_MIXED_COMP).
__global__ void __launch_bounds__(CD_TPB) k_cd_rows_comp(int64_t n, const int64_t *rowptr, const int32_t *colidx,
                                                       const float *vals, const __nv_bfloat16 *res,
                                                       const float2 *Uk, double *V, double *cV, double *A,
                                                       const double *C, const double *invMC, double dt_2, CdLoad ld)
{
    int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / CD_LANES;
    const int sub = threadIdx.x & (CD_LANES - 1);
    const unsigned mask = 0xffffffffu;
    float s = 0.f, c = 0.f;
    if (row < n) {
        for (int64_t k = rowptr[row] + sub; k < rowptr[row + 1]; k += CD_LANES) acc_pair(s, c, vals[k], __bfloat162float(res[k]), Uk[colidx[k]]);
    }
#pragma unroll
    for (int o = CD_LANES / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(mask, s, o), c2 = __shfl_xor_sync(mask, c, o);
        add_pair(s, c, s2, c2);
    }
    if (row < n && sub == 0) {
        const double sv = (double)s + (double)c;
        double a = A[row], v = V[row], cv = cV[row];
        double f = ld.at(row);
        f -= sv + C[row] * (v + dt_2 * a);
        kahan_add(v, cv, dt_2 * a);
        a = invMC[row] * f;
        kahan_add(v, cv, dt_2 * a);
        A[row] = a;
        V[row] = v;
        cV[row] = cv;
    }
}

// block (node r, neighbour slot s), entry (i, j) = K[dof(r,i), dof(nbr,j)]
// (zero where either dof is excluded or the matrix has no entry), found by
// binary search in the sorted CSR row; one warp per node
template <class VT>
__global__ void k_bsr_fill(int64_t nnodes, int64_t n, const int32_t *dof, const int64_t *rowptr,
                           const int32_t *colidx, const double *vals, const int64_t *nbr_off, const int32_t *nbr,
                           VT *blk)
{
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= nnodes) return;
    const int64_t off = nbr_off[r];
    const int ns = (int)(nbr_off[r + 1] - off);
    for (int idx = lane; idx < ns * 36; idx += 32) {
        const int sl = idx / 36, ij = idx - 36 * sl, i = ij / 6, j = ij - 6 * i;
        const int32_t d = dof[(int64_t)i * nnodes + r];
        const int32_t e = dof[(int64_t)j * nnodes + nbr[off + sl]];
        double v = 0.0;
        if (d <= n && e <= n) {
            int64_t lo = rowptr[d - 1], hi = rowptr[d] - 1;
            while (lo <= hi) {
                const int64_t mid = (lo + hi) >> 1;
                const int32_t cc = colidx[mid];
                if (cc == e - 1) {
                    v = vals[mid];
                    break;
                }
                if (cc < e - 1) lo = mid + 1; else hi = mid - 1;
            }
        }
        blk[(off + sl) * 36 + ij] = (VT)v;
    }
}

// float values and their bf16 residuals: hi = float(v), res = v - hi
__device__ __forceinline__ void split_value(double v, float &hi, __nv_bfloat16 &res)
{
    hi = (float)v;
    res = __float2bfloat16_rn((float)(v - (double)hi));
}

// the block form of k_bsr_fill with float values and bf16 residuals
__global__ void k_bsr_fill_split(int64_t nnodes, int64_t n, const int32_t *dof, const int64_t *rowptr,
                                 const int32_t *colidx, const double *vals, const int64_t *nbr_off, const int32_t *nbr,
                                 float *blk, __nv_bfloat16 *res)
{
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= nnodes) return;
    const int64_t off = nbr_off[r];
    const int ns = (int)(nbr_off[r + 1] - off);
    for (int idx = lane; idx < ns * 36; idx += 32) {
        const int sl = idx / 36, ij = idx - 36 * sl, i = ij / 6, j = ij - 6 * i;
        const int32_t d = dof[(int64_t)i * nnodes + r];
        const int32_t e = dof[(int64_t)j * nnodes + nbr[off + sl]];
        double v = 0.0;
        if (d <= n && e <= n) {
            int64_t lo = rowptr[d - 1], hi = rowptr[d] - 1;
            while (lo <= hi) {
                const int64_t mid = (lo + hi) >> 1;
                const int32_t cc = colidx[mid];
                if (cc == e - 1) {
                    v = vals[mid];
                    break;
                }
                if (cc < e - 1) lo = mid + 1; else hi = mid - 1;
            }
        }
        split_value(v, blk[(off + sl) * 36 + ij], res[(off + sl) * 36 + ij]);
    }
}

__global__ void k_split_values(int64_t n, const double *src, float *hi, __nv_bfloat16 *res)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) split_value(src[i], hi[i], res[i]);
}

__global__ void k_pad_map(int64_t nnodes, int64_t n, const int32_t *dof, int32_t *pad_of_dof)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 6 * nnodes) return;
    const int64_t r = q / 6;
    const int k = (int)(q - 6 * r);
    const int32_t d = dof[(int64_t)k * nnodes + r];
    if (d <= n) pad_of_dof[d - 1] = (int32_t)q;
}

static int enqueue_steps(fs_ctx *c, int64_t nsteps)
{
    auto &x = c->ex;
    int64_t n = x.n;
    double dt = x.dt;
    CdLoad ld{x.load ? x.Fmag : nullptr, x.mul, x.nmul, x.step, 0};
    unsigned g1 = (unsigned)((n + CD_TPB - 1) / CD_TPB);
    unsigned g2 = (unsigned)((n * CD_LANES + CD_TPB - 1) / CD_TPB);
    if (x.bsr) {
        const unsigned gb = (unsigned)((x.nnodes + 39) / 40);  // 5 nodes per warp, 8 warps per block
        for (int64_t s = 0; s < nsteps; s++) {
            ld.j = (int)s;
            if (x.precision == FS_FP64) {
                k_cd_disp_pad<double><<<g1, CD_TPB, 0, c->stream>>>(n, dt, dt * dt / 2, x.U, x.cU, x.V, x.A,
                                                                     x.pad_of_dof, (double *)x.xp);
                k_cd_bsr<double><<<gb, CD_TPB, 0, c->stream>>>(x.nnodes, n, c->mesh.dof, c->pat.nbr_off,
                                                                c->pat.nbr, (const double *)x.blk,
                                                                (const double *)x.xp, x.V, x.cV, x.A, x.C,
                                                                x.invMC, dt / 2, ld);
            } else if (x.precision == FS_MIXED_COMP) {
                k_cd_disp_pad<float2><<<g1, CD_TPB, 0, c->stream>>>(n, dt, dt * dt / 2, x.U, x.cU, x.V, x.A,
                                                                     x.pad_of_dof, (float2 *)x.xp);
                k_cd_bsr_comp<<<gb, CD_TPB, 0, c->stream>>>(x.nnodes, n, c->mesh.dof, c->pat.nbr_off, c->pat.nbr,
                                                             (const float *)x.blk, (const __nv_bfloat16 *)x.res,
                                                             (const float2 *)x.xp, x.V, x.cV, x.A, x.C, x.invMC,
                                                             dt / 2, ld);
            } else {
                k_cd_disp_pad<float><<<g1, CD_TPB, 0, c->stream>>>(n, dt, dt * dt / 2, x.U, x.cU, x.V, x.A,
                                                                    x.pad_of_dof, (float *)x.xp);
                k_cd_bsr<float><<<gb, CD_TPB, 0, c->stream>>>(x.nnodes, n, c->mesh.dof, c->pat.nbr_off,
                                                               c->pat.nbr, (const float *)x.blk,
                                                               (const float *)x.xp, x.V, x.cV, x.A, x.C,
                                                               x.invMC, dt / 2, ld);
            }
        }
        if (x.load && nsteps > 0) k_step_advance<<<1, 1, 0, c->stream>>>(x.step, nsteps);
        return cuda_check(c, cudaGetLastError(), "explicit step launch");
    }
    for (int64_t s = 0; s < nsteps; s++) {
        ld.j = (int)s;
        if (x.precision == FS_MIXED_COMP) {
            k_cd_disp_pair<<<g1, CD_TPB, 0, c->stream>>>(n, dt, dt * dt / 2, x.U, x.cU, x.V, x.A, (float2 *)x.U32);
            k_cd_rows_comp<<<g2, CD_TPB, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, x.vals32,
                                                          (const __nv_bfloat16 *)x.res, (const float2 *)x.U32, x.V,
                                                          x.cV, x.A, x.C, x.invMC, dt / 2, ld);
            continue;
        }
        bool single = x.precision != FS_FP64;
        k_cd_disp<<<g1, CD_TPB, 0, c->stream>>>(n, dt, dt * dt / 2, x.U, x.cU, x.V, x.A, single ? x.U32 : nullptr);
        if (!single)
            k_cd_rows<double><<<g2, CD_TPB, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, c->vals, x.U, x.V,
                                                            x.cV, x.A, x.C, x.invMC, dt / 2, ld);
        else
            k_cd_rows<float><<<g2, CD_TPB, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, x.vals32, x.U32, x.V,
                                                           x.cV, x.A, x.C, x.invMC, dt / 2, ld);
    }
    if (x.load && nsteps > 0) k_step_advance<<<1, 1, 0, c->stream>>>(x.step, nsteps);
    return cuda_check(c, cudaGetLastError(), "explicit step launch");
}

int explicit_launch_steps(fs_ctx *c, int64_t nsteps)
{
    auto &x = c->ex;
    if (nsteps <= 0) return FS_OK;
    if (!x.exec) {
        FS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int st = enqueue_steps(c, CD_GRAPH_STEPS);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (st != FS_OK) return st;
        FS_CUDA(c, e);
        x.graph = g;
        FS_CUDA(c, cudaGraphInstantiate(&x.exec, g, 0));
        x.graph_steps = CD_GRAPH_STEPS;
    }
    int64_t full = nsteps / x.graph_steps, rest = nsteps % x.graph_steps;
    for (int64_t k = 0; k < full; k++) FS_CUDA(c, cudaGraphLaunch(x.exec, c->stream));
    FS_TRY(enqueue_steps(c, rest));
    return FS_OK;
}

__global__ void k_to_float(int64_t n, const double *src, float *dst)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

// ---------------------------------------------------------------------------
// power iteration for the largest generalized eigenvalue of (K, M), M
// diagonal: the reference's `pwr` (clamp_cyl_expl_examples.jl:131-142),
// w = K v / |K v|, v = M^-1 w / |M^-1 w|, omega = sqrt(v'Kv / v'Mv).
// Reductions are two-pass with a fixed order: bitwise reproducible.
// ---------------------------------------------------------------------------
static const int PI_TPB = 256;
static const int PI_BLOCKS = 1024;

// y = alpha K x, CD_LANES lanes per row
__global__ void k_spmv(int64_t n, const int64_t *rowptr, const int32_t *colidx, const double *vals,
                       const double *x, double *y, double alpha = 1.0)
{
    int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / CD_LANES;
    const int sub = threadIdx.x & (CD_LANES - 1);
    double s = 0.0;
    if (row < n)
        for (int64_t k = rowptr[row] + sub; k < rowptr[row + 1]; k += CD_LANES) s += vals[k] * x[colidx[k]];
#pragma unroll
    for (int o = CD_LANES / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (row < n && sub == 0) y[row] = alpha * s;
}

// partial[b] = sum over this block's strided range of a[i] * b[i] (b may be a weight)
__global__ void k_dot_partial(int64_t n, const double *a, const double *b, double *partial)
{
    __shared__ double sh[PI_TPB];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * PI_TPB + threadIdx.x; i < n; i += (int64_t)PI_BLOCKS * PI_TPB)
        s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = PI_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(const double *partial, double *out)
{
    __shared__ double sh[PI_TPB];
    double s = 0.0;
    for (int i = threadIdx.x; i < PI_BLOCKS; i += PI_TPB) s += partial[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = PI_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// y = x * (1/sqrt(*nrm2)) * (w ? w[i] : 1)
__global__ void k_scale(int64_t n, const double *x, const double *nrm2, const double *w, double *y)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f = 1.0 / sqrt(*nrm2);
    y[i] = x[i] * f * (w ? w[i] : 1.0);
}

// deterministic start vector in [0, 1) from a 64-bit mix of (seed, i)
__global__ void k_start(int64_t n, uint64_t seed, double *v)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z = z ^ (z >> 31);
    v[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

void end_explicit(fs_ctx *c)
{
    auto &x = c->ex;
    if (x.exec) cudaGraphExecDestroy(x.exec);
    if (x.graph) cudaGraphDestroy(x.graph);
    x.exec = nullptr;
    x.graph = nullptr;
    x.ready = false;
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_power_iteration(fs_ctx *c, const double *mdiag, int64_t iters, uint64_t seed, double *omega_max)
{
    if (!c || !mdiag || !omega_max || iters < 1) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_last_stiffness(c));
    int64_t n = c->mat_n;
    if (n == 0) return set_err(c, FS_ERR_BAD_INPUT, "empty matrix");
    size_t need = sizeof(double) * (size_t)(4 * n + PI_BLOCKS + 4);
    FS_TRY(ensure_scratch(c, need));
    double *v = (double *)c->scratch, *w = v + n, *minv = w + n, *md = minv + n;
    double *partial = md + n, *red = partial + PI_BLOCKS;
    FS_CUDA(c, cudaMemcpyAsync(md, mdiag, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    unsigned g = (unsigned)((n + 255) / 256), gs = (unsigned)((n * CD_LANES + 255) / 256);
    std::vector<double> h((size_t)n);
    for (int64_t i = 0; i < n; i++) h[i] = 1.0 / mdiag[i];
    FS_CUDA(c, cudaMemcpyAsync(minv, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    k_start<<<g, 256, 0, c->stream>>>(n, seed, v);
    for (int64_t it = 0; it < iters; it++) {
        k_spmv<<<gs, 256, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, c->vals, v, w);
        k_dot_partial<<<PI_BLOCKS, PI_TPB, 0, c->stream>>>(n, w, w, partial);
        k_dot_final<<<1, PI_TPB, 0, c->stream>>>(partial, red);
        k_scale<<<g, 256, 0, c->stream>>>(n, w, red, minv, v);       // v = M^-1 w / |w|
        k_dot_partial<<<PI_BLOCKS, PI_TPB, 0, c->stream>>>(n, v, v, partial);
        k_dot_final<<<1, PI_TPB, 0, c->stream>>>(partial, red);
        k_scale<<<g, 256, 0, c->stream>>>(n, v, red, nullptr, v);    // v = v / |v|
    }
    // Rayleigh quotient v'Kv / v'Mv
    double one = 1.0;
    FS_CUDA(c, cudaMemcpyAsync(red + 3, &one, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_spmv<<<gs, 256, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, c->vals, v, w);
    k_dot_partial<<<PI_BLOCKS, PI_TPB, 0, c->stream>>>(n, v, w, partial);
    k_dot_final<<<1, PI_TPB, 0, c->stream>>>(partial, red + 1);
    k_scale<<<g, 256, 0, c->stream>>>(n, v, red + 3, md, w);  // w = m .* v
    k_dot_partial<<<PI_BLOCKS, PI_TPB, 0, c->stream>>>(n, v, w, partial);
    k_dot_final<<<1, PI_TPB, 0, c->stream>>>(partial, red + 2);
    FS_CUDA(c, cudaGetLastError());
    double hr[2];
    FS_CUDA(c, cudaMemcpyAsync(hr, red + 1, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    *omega_max = sqrt(hr[0] / hr[1]);
    return FS_OK;
}

int fs_explicit_setup(fs_ctx *c, int precision, const double *invMC, const double *C, double dt)
{
    if (!c || !invMC || !C) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_last_stiffness(c));
    if (precision != FS_FP64 && precision != FS_MIXED && precision != FS_MIXED_COMP)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown precision");
    if (!(dt > 0.0)) return set_err(c, FS_ERR_BAD_INPUT, "time step must be positive");
    auto &x = c->ex;
    if (x.exec) cudaGraphExecDestroy(x.exec);
    if (x.graph) cudaGraphDestroy(x.graph);
    x.exec = nullptr;
    x.graph = nullptr;
    x.load = false;
    int64_t n = c->mat_n;
    x.n = n;
    x.dt = dt;
    x.precision = precision;
    FS_TRY(dalloc(c, &x.U, (size_t)n)); FS_TRY(dalloc(c, &x.V, (size_t)n)); FS_TRY(dalloc(c, &x.A, (size_t)n));
    FS_TRY(dalloc(c, &x.cU, (size_t)n)); FS_TRY(dalloc(c, &x.cV, (size_t)n));
    FS_TRY(dalloc(c, &x.invMC, (size_t)n)); FS_TRY(dalloc(c, &x.C, (size_t)n));
    size_t bn = sizeof(double) * (size_t)std::max<int64_t>(n, 1);
    FS_CUDA(c, cudaMemsetAsync(x.U, 0, bn, c->stream));
    FS_CUDA(c, cudaMemsetAsync(x.V, 0, bn, c->stream));
    FS_CUDA(c, cudaMemsetAsync(x.A, 0, bn, c->stream));
    FS_CUDA(c, cudaMemsetAsync(x.cU, 0, bn, c->stream));
    FS_CUDA(c, cudaMemsetAsync(x.cV, 0, bn, c->stream));
    FS_CUDA(c, cudaMemcpyAsync(x.invMC, invMC, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    FS_CUDA(c, cudaMemcpyAsync(x.C, C, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    // 6x6 node-block form when the pattern of the current mesh is there (its
    // neighbour lists are the block rows); otherwise the CSR product
    x.bsr = c->pat.n >= 0 && c->pat.nbr_off && c->mesh.nnodes > 0;
    if (x.bsr) {
        const MeshDev &m = c->mesh;
        const int64_t nn = m.nnodes;
        int64_t nbr_total = 0;
        FS_CUDA(c, cudaMemcpyAsync(&nbr_total, c->pat.nbr_off + nn, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
        // block values: double or float; displacement copy: double, float,
        // or float pairs (FS_MIXED_COMP)
        const size_t es = precision == FS_FP64 ? 8 : 4, xs = precision == FS_MIXED ? 4 : 8;
        dfree(&x.blk);
        dfree(&x.xp);
        FS_CUDA(c, cudaMalloc(&x.blk, es * 36 * (size_t)std::max<int64_t>(nbr_total, 1)));
        FS_CUDA(c, cudaMalloc(&x.xp, xs * 6 * (size_t)nn));
        FS_CUDA(c, cudaMemsetAsync(x.xp, 0, xs * 6 * (size_t)nn, c->stream));
        FS_TRY(dalloc(c, &x.pad_of_dof, (size_t)n));
        FS_CUDA(c, cudaMemsetAsync(x.pad_of_dof, 0xff, sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1), c->stream));
        k_pad_map<<<(unsigned)((6 * nn + 255) / 256), 256, 0, c->stream>>>(nn, n, m.dof, x.pad_of_dof);
        const unsigned gw = (unsigned)((nn * 32 + 255) / 256);
        dfree(&x.res);
        if (precision == FS_FP64)
            k_bsr_fill<double><<<gw, 256, 0, c->stream>>>(nn, n, m.dof, c->mat_rowptr, c->mat_colidx, c->vals,
                                                           c->pat.nbr_off, c->pat.nbr, (double *)x.blk);
        else if (precision == FS_MIXED_COMP) {
            FS_CUDA(c, cudaMalloc(&x.res, 2 * 36 * (size_t)std::max<int64_t>(nbr_total, 1)));
            k_bsr_fill_split<<<gw, 256, 0, c->stream>>>(nn, n, m.dof, c->mat_rowptr, c->mat_colidx, c->vals,
                                                         c->pat.nbr_off, c->pat.nbr, (float *)x.blk,
                                                         (__nv_bfloat16 *)x.res);
        } else
            k_bsr_fill<float><<<gw, 256, 0, c->stream>>>(nn, n, m.dof, c->mat_rowptr, c->mat_colidx, c->vals,
                                                          c->pat.nbr_off, c->pat.nbr, (float *)x.blk);
        FS_CUDA(c, cudaGetLastError());
        x.nnodes = nn;
    } else if (precision != FS_FP64) {
        // float copy of U, or float pairs (two floats a dof) for FS_MIXED_COMP
        FS_TRY(dalloc(c, &x.U32, (size_t)n * (precision == FS_MIXED_COMP ? 2 : 1)));
        FS_TRY(dalloc(c, &x.vals32, (size_t)c->mat_nnz));
        dfree(&x.res);
        if (precision == FS_MIXED_COMP) {
            FS_CUDA(c, cudaMalloc(&x.res, 2 * (size_t)std::max<int64_t>(c->mat_nnz, 1)));
            if (c->mat_nnz)
                k_split_values<<<(unsigned)((c->mat_nnz + 255) / 256), 256, 0, c->stream>>>(
                    c->mat_nnz, c->vals, x.vals32, (__nv_bfloat16 *)x.res);
        } else if (c->mat_nnz)
            k_to_float<<<(unsigned)((c->mat_nnz + 255) / 256), 256, 0, c->stream>>>(c->mat_nnz, c->vals, x.vals32);
        FS_CUDA(c, cudaGetLastError());
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    x.ready = true;
    return FS_OK;
}

int fs_explicit_set_state(fs_ctx *c, const double *U, const double *V, const double *A)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    auto &x = c->ex;
    if (!x.ready) return set_err(c, FS_ERR_STATE, "call fs_explicit_setup first");
    size_t bn = sizeof(double) * (size_t)x.n;
    if (U) FS_CUDA(c, cudaMemcpyAsync(x.U, U, bn, cudaMemcpyHostToDevice, c->stream));
    if (V) FS_CUDA(c, cudaMemcpyAsync(x.V, V, bn, cudaMemcpyHostToDevice, c->stream));
    if (A) FS_CUDA(c, cudaMemcpyAsync(x.A, A, bn, cudaMemcpyHostToDevice, c->stream));
    if (bn) {
        FS_CUDA(c, cudaMemsetAsync(x.cU, 0, bn, c->stream));
        FS_CUDA(c, cudaMemsetAsync(x.cV, 0, bn, c->stream));
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_explicit_set_load(fs_ctx *c, const double *Fmag, const double *mul, int64_t nmul, int64_t step0)
{
    if (!c || nmul < 0 || step0 < 0) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    auto &x = c->ex;
    if (!x.ready) return set_err(c, FS_ERR_STATE, "call fs_explicit_setup first");
    if (Fmag && nmul > 0 && !mul) return set_err(c, FS_ERR_BAD_INPUT, "missing time function values");
    // the captured steps hold the load pointers: capture again on the next run
    if (x.exec) cudaGraphExecDestroy(x.exec);
    if (x.graph) cudaGraphDestroy(x.graph);
    x.exec = nullptr;
    x.graph = nullptr;
    x.load = Fmag != nullptr;
    if (!x.load) return FS_OK;
    FS_TRY(grow(c, &x.Fmag, &x.cap_Fmag, (size_t)std::max<int64_t>(x.n, 1)));
    FS_TRY(grow(c, &x.mul, &x.cap_mul, (size_t)std::max<int64_t>(nmul, 1)));
    if (!x.step) FS_TRY(dalloc(c, &x.step, 1));
    x.nmul = nmul;
    FS_CUDA(c, cudaMemcpyAsync(x.Fmag, Fmag, sizeof(double) * (size_t)x.n, cudaMemcpyHostToDevice, c->stream));
    if (nmul) FS_CUDA(c, cudaMemcpyAsync(x.mul, mul, sizeof(double) * (size_t)nmul, cudaMemcpyHostToDevice, c->stream));
    FS_CUDA(c, cudaMemcpyAsync(x.step, &step0, sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_explicit_run(fs_ctx *c, int64_t nsteps)
{
    if (!c || nsteps < 0) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (!c->ex.ready) return set_err(c, FS_ERR_STATE, "call fs_explicit_setup first");
    FS_TRY(explicit_launch_steps(c, nsteps));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_explicit_get_state(fs_ctx *c, double *U, double *V, double *A)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    auto &x = c->ex;
    if (!x.ready) return set_err(c, FS_ERR_STATE, "call fs_explicit_setup first");
    size_t bn = sizeof(double) * (size_t)x.n;
    if (U) FS_CUDA(c, cudaMemcpyAsync(U, x.U, bn, cudaMemcpyDeviceToHost, c->stream));
    if (V) FS_CUDA(c, cudaMemcpyAsync(V, x.V, bn, cudaMemcpyDeviceToHost, c->stream));
    if (A) FS_CUDA(c, cudaMemcpyAsync(A, x.A, bn, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

// Restoring force of the shells: -K U with the last assembled matrix.
int fs_restoring_force(fs_ctx *c, const double *U, double *F)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_last_stiffness(c));
    const int64_t n = c->mat_n;
    if (n && (!U || !F)) return set_err(c, FS_ERR_BAD_INPUT, "missing vector");
    if (n == 0) return FS_OK;
    FS_TRY(ensure_scratch(c, sizeof(double) * 2 * (size_t)n));
    double *u = (double *)c->scratch, *f = u + n;
    FS_CUDA(c, cudaMemcpyAsync(u, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    const unsigned gs = (unsigned)((n * CD_LANES + 255) / 256);
    k_spmv<<<gs, 256, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, c->vals, u, f, -1.0);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaMemcpyAsync(F, f, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // extern "C"

// Test-only device build of the compensated sums (csrc/fs_comp_sum.cuh): the
// same dot products and float-triple column sums as tests/hostcheck, one
// input per thread, so that the packed FP32x2 instructions can be compared
// bitwise with the host's lane-by-lane IEEE arithmetic.  Not part of the
// product.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_comp_sum.cuh"

using namespace fs;

// m dot products of length n: (a_t . b0_t, a_t . b1_t) at `levels` levels,
// out[4 t ..] = {hi0, lo0, hi1, lo1}
__global__ void k_comp_dot(int levels, int n, int m, const float *a, const float *b0, const float *b1,
                           float *out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const float *at = a + (int64_t)n * t, *b0t = b0 + (int64_t)n * t, *b1t = b1 + (int64_t)n * t;
    f32x2 s = x2_pack(0.f, 0.f), c = s, d = s, hh, ll;
    for (int r = 0; r < n; r++) {
        const f32x2 a2 = x2_pack(at[r], at[r]), na2 = x2_pack(-at[r], -at[r]), b2 = x2_pack(b0t[r], b1t[r]);
        if (levels == 3)
            dot3_step_x2(s, c, d, a2, na2, b2);
        else
            dot2_step_x2(s, c, a2, na2, b2);
    }
    if (levels == 3)
        x2_pair_finish<3>(s, c, d, hh, ll);
    else
        x2_pair_finish<2>(s, c, d, hh, ll);
    x2_unpack(hh, out[4 * t], out[4 * t + 2]);
    x2_unpack(ll, out[4 * t + 1], out[4 * t + 3]);
}

// m column sums of n float pairs on both lanes: lane k of sum t sums
// (hi[(2 t + k) n + r], lo[(2 t + k) n + r]), r < n; out[2 t + k]
__global__ void k_triple_sum(int n, int m, const float *hi, const float *lo, double *out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const float *h0 = hi + (int64_t)2 * n * t, *l0 = lo + (int64_t)2 * n * t;
    f32x2 h = x2_pack(h0[0], h0[n]), l = x2_pack(l0[0], l0[n]), tl = x2_pack(0.f, 0.f);
    for (int r = 1; r < n; r++) x2_triple_add(h, l, tl, x2_pack(h0[r], h0[n + r]), x2_pack(l0[r], l0[n + r]));
    float a0, a1, b0, b1, c0, c1;
    x2_unpack(h, a0, a1);
    x2_unpack(l, b0, b1);
    x2_unpack(tl, c0, c1);
    out[2 * t] = triple_value(a0, b0, c0);
    out[2 * t + 1] = triple_value(a1, b1, c1);
}

template <class T> static int to_device(T **d, const T *h, size_t count)
{
    if (cudaMalloc(d, count * sizeof(T)) != cudaSuccess) return 1;
    if (h && cudaMemcpy(*d, h, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return 1;
    return 0;
}

extern "C" int dc_comp_dot(int levels, int n, int m, const float *a, const float *b0, const float *b1, float *out)
{
    if ((levels != 2 && levels != 3) || n < 1 || m < 1) return 1;
    float *da = nullptr, *db0 = nullptr, *db1 = nullptr, *dout = nullptr;
    const size_t nm = (size_t)n * m;
    int st = to_device(&da, a, nm) || to_device(&db0, b0, nm) || to_device(&db1, b1, nm) ||
             to_device(&dout, (const float *)nullptr, (size_t)4 * m);
    if (!st) {
        k_comp_dot<<<(m + 127) / 128, 128>>>(levels, n, m, da, db0, db1, dout);
        st = cudaGetLastError() != cudaSuccess ||
             cudaMemcpy(out, dout, (size_t)4 * m * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess;
    }
    cudaFree(da);
    cudaFree(db0);
    cudaFree(db1);
    cudaFree(dout);
    return st ? 2 : 0;
}

extern "C" int dc_triple_sum(int n, int m, const float *hi, const float *lo, double *out)
{
    if (n < 1 || m < 1) return 1;
    float *dh = nullptr, *dl = nullptr;
    double *dout = nullptr;
    const size_t cnt = (size_t)2 * n * m;
    int st = to_device(&dh, hi, cnt) || to_device(&dl, lo, cnt) ||
             to_device(&dout, (const double *)nullptr, (size_t)2 * m);
    if (!st) {
        k_triple_sum<<<(m + 127) / 128, 128>>>(n, m, dh, dl, dout);
        st = cudaGetLastError() != cudaSuccess ||
             cudaMemcpy(out, dout, (size_t)2 * m * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess;
    }
    cudaFree(dh);
    cudaFree(dl);
    cudaFree(dout);
    return st ? 2 : 0;
}

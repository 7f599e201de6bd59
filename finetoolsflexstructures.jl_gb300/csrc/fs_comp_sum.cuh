// Compensated float arithmetic of the FS_MIXED_COMP mode: two floats in one
// 64-bit register pair (f32x2), the error-free transformations on them, the
// element kernels' compensated dot products and the gather's float-triple
// sums.
//
// Under nvcc the operations are the packed FP32x2 instructions of the
// sm_100 family (add/sub/mul/fma .rn .f32x2), both halves rounded to nearest
// as the scalar instructions round them.  Any other compiler gets the same
// operations lane by lane in IEEE binary32 arithmetic (build it without
// floating-point contraction: -ffp-contract=off), so the sums can be run and
// checked on a host.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define FS_X2 __device__ __forceinline__
#else
#include <cmath>
#define FS_X2 inline
#endif

namespace fs {

// Gram sums per element type in FS_MIXED_COMP: a T3 entry sums at most 9
// rows (Dot2: two levels), a Q4 entry at most 33 (three levels).
constexpr int T3_PAIR_LEVELS = 2;
constexpr int Q4_PAIR_LEVELS = 3;

#if defined(__CUDACC__)
typedef unsigned long long f32x2;
FS_X2 f32x2 x2_pack(float lo, float hi)
{
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
FS_X2 void x2_unpack(f32x2 v, float &lo, float &hi) { asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v)); }
FS_X2 f32x2 x2_add(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
FS_X2 f32x2 x2_sub(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
FS_X2 f32x2 x2_mul(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
FS_X2 f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
#else
struct f32x2 {
    float lo, hi;
};
FS_X2 f32x2 x2_pack(float lo, float hi) { return f32x2{lo, hi}; }
FS_X2 void x2_unpack(f32x2 v, float &lo, float &hi)
{
    lo = v.lo;
    hi = v.hi;
}
FS_X2 f32x2 x2_add(f32x2 a, f32x2 b) { return f32x2{a.lo + b.lo, a.hi + b.hi}; }
FS_X2 f32x2 x2_sub(f32x2 a, f32x2 b) { return f32x2{a.lo - b.lo, a.hi - b.hi}; }
FS_X2 f32x2 x2_mul(f32x2 a, f32x2 b) { return f32x2{a.lo * b.lo, a.hi * b.hi}; }
FS_X2 f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c)
{
    return f32x2{std::fma(a.lo, b.lo, c.lo), std::fma(a.hi, b.hi, c.hi)};
}
#endif

// s + v by TwoSum (Knuth): s <- fl(s + v), returns the exact error
FS_X2 f32x2 x2_two_sum(f32x2 &s, f32x2 v)
{
    const f32x2 t = x2_add(s, v);
    const f32x2 z = x2_sub(t, s);
    const f32x2 e = x2_add(x2_sub(s, x2_sub(t, z)), x2_sub(v, z));
    s = t;
    return e;
}

// One step of a three-level compensated dot product on two entries at once
// (the error-free transformations of Ogita, Rump and Oishi's Dot2, applied
// once more to the compensation term): the product a b split exactly into p
// and pl (m = fma(-a, b, p) = -pl exactly), p added to s by TwoSum (error e),
// e added to c by TwoSum (error f), and f + pl added to d.  What is lost is
// the rounding of d's terms, about 2^-24 of |d|, itself of the order of
// 2^-24 of the sum of |a b|: after n terms at most about 2 n 2^-48 of that
// sum, against Dot2's n^2 2^-48.
FS_X2 void dot3_step_x2(f32x2 &s, f32x2 &c, f32x2 &d, f32x2 a, f32x2 na, f32x2 b)
{
    const f32x2 p = x2_mul(a, b);
    const f32x2 m = x2_fma(na, b, p);
    const f32x2 e = x2_two_sum(s, p);
    const f32x2 f = x2_two_sum(c, e);
    d = x2_add(d, x2_sub(f, m));
}

// Dot2 on two entries at once: the product split exactly, p added to s by
// TwoSum, its error and the product's (e + pl = e - m) added to c.
FS_X2 void dot2_step_x2(f32x2 &s, f32x2 &c, f32x2 a, f32x2 na, f32x2 b)
{
    const f32x2 p = x2_mul(a, b);
    const f32x2 m = x2_fma(na, b, p);
    const f32x2 e = x2_two_sum(s, p);
    c = x2_add(c, x2_sub(e, m));
}

// The (hi, lo) float pairs of a compensated dot product: the compensation
// (c + d with three levels, c with two) rounded below the pair's last bit,
// then Fast2Sum with s, exact while |s| is at least the compensation's
// magnitude.
template <int LEVELS> FS_X2 void x2_pair_finish(f32x2 s, f32x2 c, f32x2 d, f32x2 &hh, f32x2 &ll)
{
    const f32x2 cd = LEVELS == 3 ? x2_add(c, d) : c;
    hh = x2_add(s, cd);
    ll = x2_sub(cd, x2_sub(hh, s));
}

#if defined(__CUDACC__)
// exact float -> double built from the bit pattern with integer operations
// only (zeros, subnormals, normals, inf and nan), so that no conversion
// lands on the double-precision pipe
FS_X2 double f2d_exact(float f)
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
FS_X2 double f2d_fast(float f)
{
    const uint32_t u = __float_as_uint(f), a = u & 0x7fffffffu;
    if (a != 0u && a - 0x00800000u >= 0x7f000000u) return f2d_exact(f);  // subnormal, inf, nan
    const uint32_t h = (u & 0x80000000u) | (a != 0u ? (a >> 3) + 0x38000000u : 0u);
    return __hiloint2double((int)h, (int)(u << 29));
}
#else
FS_X2 double f2d_fast(float f) { return (double)f; }
#endif

// The gather's sum of float pairs (hi + lo each) as an unevaluated float
// triple: the pair's low half into the low part, its high half into the
// high part and that error into the low part, both errors of the low part
// added to the tail.  What is lost is the tail's rounding, of the order of
// 2^-72 of the summed magnitudes per term.
FS_X2 void x2_triple_add(f32x2 &hi, f32x2 &lo, f32x2 &tl, f32x2 vhi, f32x2 vlo)
{
    const f32x2 f0 = x2_two_sum(lo, vlo);
    const f32x2 f1 = x2_two_sum(lo, x2_two_sum(hi, vhi));
    tl = x2_add(tl, x2_add(f0, f1));
}

// One lane of a float triple rounded to double: lo + tl in double (exact
// while their exponents are within 29 of each other), then hi added with one
// rounding, 2^-53 of the value.
FS_X2 double triple_value(float h, float l, float t)
{
    double v = f2d_fast(h);
    if (l != 0.f || t != 0.f) v += f2d_fast(l) + f2d_fast(t);
    return v;
}

}  // namespace fs

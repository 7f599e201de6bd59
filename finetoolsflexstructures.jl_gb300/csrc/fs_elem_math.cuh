// Per-element math of the shell hot path, shared by the CUDA kernels (and,
// for checking, by a host build of the same header).
//
// Formulation.  The reference (FinEtoolsFlexStructures.jl 3.6.4) builds the
// element matrix in the element frame and then applies two dense 18x18 /
// 24x24 congruences (src/FEMMShellT3FFModule.jl:708-730,
// src/FEMMShellQ4RSModule.jl:925-936).  Here the same matrix is written as a
// Gram product K = Bh^T Bh, where every row of Bh is one strain component
// already expressed on the GLOBAL dofs:
//
//   * the element-frame strain-displacement rows (membrane, bending,
//     transverse shear) are combined with the Cholesky factor of the
//     material matrix (D = L L^T) and the quadrature weight, and
//   * the nodal-to-element transformation (triads, drilling coupling
//     1/2 (v,x - u,y) of src/FEMMShellT3FFModule.jl:421-463) and the
//     global-to-nodal rotation are folded into each row analytically,
//   * the drilling penalty kavg * (n . theta)^2 becomes one extra row per
//     node with a valid normal.
//
// Mathematically this is identical to the reference; numerically it differs
// by rounding only.  Geometry (element frame, nodal triads, the drilling
// factor) is always computed in double; the strain rows and the Gram product
// use the template precision R (double for the FP64 path, float for the
// mixed path).
#pragma once
#include <math.h>
#include <stdint.h>

#ifndef FS_HD
#if defined(__CUDACC__)
#define FS_HD __host__ __device__ __forceinline__
#else
#define FS_HD inline
#endif
#endif

namespace fs {

// ---------------------------------------------------------------------------
// small vector helpers
// ---------------------------------------------------------------------------
template <class T> FS_HD T dot3(const T a[3], const T b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

template <class T> FS_HD void cross3(const T a[3], const T b[3], T c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

FS_HD double rsqrt_d(double x)
{
#if defined(__CUDA_ARCH__)
    return rsqrt(x);
#else
    return 1.0 / sqrt(x);
#endif
}

// Element frame from two tangents (reference _e_g!, src/FEMMShellT3FFModule.jl:283-305):
// e1 = a/|a|, e3 = (e1 x b)/|e1 x b|, e2 = e3 x e1.  e[k][c] = component c of e_k.
FS_HD void make_frame(const double a[3], const double b[3], double e[3][3])
{
    double s = rsqrt_d(dot3(a, a));
    for (int c = 0; c < 3; c++) e[0][c] = a[c] * s;
    cross3(e[0], b, e[2]);
    s = rsqrt_d(dot3(e[2], e[2]));
    for (int c = 0; c < 3; c++) e[2][c] *= s;
    cross3(e[2], e[0], e[1]);
}

// 1/sqrt(x) rounded to nearest in float (device and host)
FS_HD float rsqrt_f(float x)
{
#if defined(__CUDA_ARCH__)
    return __frsqrt_rn(x);
#else
    return (float)(1.0 / sqrt((double)x));
#endif
}

// make_frame in float
FS_HD void make_frame_f(const float a[3], const float b[3], float e[3][3])
{
    float s = rsqrt_f(dot3(a, a));
    for (int c = 0; c < 3; c++) e[0][c] = a[c] * s;
    cross3(e[0], b, e[2]);
    s = rsqrt_f(dot3(e[2], e[2]));
    for (int c = 0; c < 3; c++) e[2][c] *= s;
    cross3(e[2], e[0], e[1]);
}

// Nodal triad (reference _NodalTriadsE, src/FEMMShellT3FFModule.jl:355-388):
// the rotation by the vector a = e3_e x n_e (angle |a|, FinEtools rotmat3!),
// in Rodrigues form R = I + s(x) [a]x + c(x) [a]x^2 with x = |a|^2,
// s = sin(phi)/phi, c = (1 - cos(phi))/phi^2.  Both are evaluated from
// their Taylor series in x (up to 9 terms: truncation below 1e-17 for x <= 1,
// fewer terms for the small angles of smooth meshes).
FS_HD void sinc_cosc(double x, double &s, double &c)
{
    if (x < 1.0e-8) {
        // truncation below x^2/5! < 1e-18
        s = 1.0 - x * (1.0 / 6.0);
        c = 0.5 - x * (1.0 / 24.0);
    } else if (x < 1.0e-4) {
        // truncation below x^4/9! < 3e-22
        s = 1.0 - x * (1.0 / 6.0 - x * (1.0 / 120.0 - x * (1.0 / 5040.0)));
        c = 0.5 - x * (1.0 / 24.0 - x * (1.0 / 720.0 - x * (1.0 / 40320.0)));
    } else if (x <= 1.0) {
        // s = sum (-x)^k/(2k+1)!,  c = sum (-x)^k/(2k+2)!
        s = 1.0 / 355687428096000.0;              // 1/17!
        s = 1.0 / 1307674368000.0 - x * s;        // 1/15!
        s = 1.0 / 6227020800.0 - x * s;           // 1/13!
        s = 1.0 / 39916800.0 - x * s;             // 1/11!
        s = 1.0 / 362880.0 - x * s;               // 1/9!
        s = 1.0 / 5040.0 - x * s;                 // 1/7!
        s = 1.0 / 120.0 - x * s;                  // 1/5!
        s = 1.0 / 6.0 - x * s;                    // 1/3!
        s = 1.0 - x * s;
        c = 1.0 / 6402373705728000.0;             // 1/18!
        c = 1.0 / 20922789888000.0 - x * c;       // 1/16!
        c = 1.0 / 87178291200.0 - x * c;          // 1/14!
        c = 1.0 / 479001600.0 - x * c;            // 1/12!
        c = 1.0 / 3628800.0 - x * c;              // 1/10!
        c = 1.0 / 40320.0 - x * c;                // 1/8!
        c = 1.0 / 720.0 - x * c;                  // 1/6!
        c = 1.0 / 24.0 - x * c;                   // 1/4!
        c = 0.5 - x * c;                          // 1/2!
    } else {
        double phi = sqrt(x);
        s = sin(phi) / phi;
        c = (1.0 - cos(phi)) / x;
    }
}

// R[r][k]: row r, column k of the triad A_E of one node.
FS_HD void nodal_triad(const double e[3][3], const double n[3], bool valid, double R[3][3])
{
    double a0 = 0.0, a1 = 0.0;
    if (valid) {
        double ne0 = dot3(e[0], n), ne1 = dot3(e[1], n);
        a0 = -ne1;
        a1 = ne0;
    }
    double x = a0 * a0 + a1 * a1;
    if (!(x > 1.0e-24)) {
        R[0][0] = 1; R[0][1] = 0; R[0][2] = 0;
        R[1][0] = 0; R[1][1] = 1; R[1][2] = 0;
        R[2][0] = 0; R[2][1] = 0; R[2][2] = 1;
        return;
    }
    double s, c;
    sinc_cosc(x, s, c);
    R[0][0] = 1.0 - c * a1 * a1; R[0][1] = c * a0 * a1;       R[0][2] = s * a1;
    R[1][0] = c * a0 * a1;       R[1][1] = 1.0 - c * a0 * a0; R[1][2] = -s * a0;
    R[2][0] = -s * a1;           R[2][1] = s * a0;            R[2][2] = 1.0 - c * x;
}

// sin(phi)/phi and (1 - cos(phi))/phi^2 in float for x = phi^2 <= 1: the
// Taylor series to x^4 (truncation below x^5/11! < 3e-8, under half an ulp
// of the results).
FS_HD void sinc_cosc_f(float x, float &s, float &c)
{
    s = 1.0f - x * (1.0f / 6.0f - x * (1.0f / 120.0f - x * (1.0f / 5040.0f - x * (1.0f / 362880.0f))));
    c = 0.5f - x * (1.0f / 24.0f - x * (1.0f / 720.0f - x * (1.0f / 40320.0f - x * (1.0f / 3628800.0f))));
}

// The triad in the working precision.  Double: nodal_triad.  Float: the
// rotation vector a = e3 x n (a difference of nearly parallel unit vectors
// on a smooth mesh) is formed in double from the double frame and rounded
// once; the Rodrigues entries are evaluated from it in float, each within
// about one float ulp of the rounded double entry.  Angles beyond one radian
// (creases) take the double path.
// The triad of the float rows from the element frame and the nodal normal,
// both rounded to float: the rotation vector, the Rodrigues entries in float
// (angles beyond one radian evaluate sin and cos in double).  The rounding of
// the frame and the normal perturbs the rows like the rounding of the rows
// themselves (it keeps K a Gram matrix).
FS_HD void nodal_triad_f(const float e[3][3], const float n[3], bool valid, float Ar[3][3])
{
    float a0 = 0.0f, a1 = 0.0f;
    if (valid) {
        a0 = -dot3(e[1], n);
        a1 = dot3(e[0], n);
    }
    const float x = a0 * a0 + a1 * a1;
    if (!(x > 1.0e-24f)) {
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 3; k++) Ar[r][k] = r == k ? 1.0f : 0.0f;
        return;
    }
    float s, c;
    if (x > 1.0f) {
        double sd, cd;
        sinc_cosc((double)x, sd, cd);
        s = (float)sd;
        c = (float)cd;
    } else {
        sinc_cosc_f(x, s, c);
    }
    const float ca0 = c * a0, ca1 = c * a1;
    Ar[0][0] = 1.0f - ca1 * a1; Ar[0][1] = ca0 * a1;       Ar[0][2] = s * a1;
    Ar[1][0] = ca0 * a1;        Ar[1][1] = 1.0f - ca0 * a0; Ar[1][2] = -(s * a0);
    Ar[2][0] = -(s * a1);       Ar[2][1] = s * a0;          Ar[2][2] = 1.0f - c * x;
}

template <class R>
FS_HD void nodal_triad_r(const double e[3][3], const double n[3], bool valid, R Ar[3][3])
{
    if constexpr (sizeof(R) == 8) {
        double A[3][3];
        nodal_triad(e, n, valid, A);
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 3; k++) Ar[r][k] = A[r][k];
    } else {
        double a0d = 0.0, a1d = 0.0;
        if (valid) {
            a0d = -dot3(e[1], n);
            a1d = dot3(e[0], n);
        }
        const float a0 = (float)a0d, a1 = (float)a1d;
        const float x = a0 * a0 + a1 * a1;
        if (!(x > 1.0e-24f)) {
            for (int r = 0; r < 3; r++)
                for (int k = 0; k < 3; k++) Ar[r][k] = r == k ? (R)1 : (R)0;
            return;
        }
        if (x > 1.0f) {
            const double xd = a0d * a0d + a1d * a1d;
            double sd, cd;
            sinc_cosc(xd, sd, cd);
            const R d0 = (R)(1.0 - cd * a1d * a1d), d1 = (R)(1.0 - cd * a0d * a0d), d2 = (R)(1.0 - cd * xd);
            const R o = (R)(cd * a0d * a1d), s1 = (R)(sd * a1d), s0 = (R)(sd * a0d);
            Ar[0][0] = d0; Ar[0][1] = o;  Ar[0][2] = s1;
            Ar[1][0] = o;  Ar[1][1] = d1; Ar[1][2] = -s0;
            Ar[2][0] = -s1; Ar[2][1] = s0; Ar[2][2] = d2;
            return;
        }
        float s, c;
        sinc_cosc_f(x, s, c);
        const float ca0 = c * a0, ca1 = c * a1;
        Ar[0][0] = 1.0f - ca1 * a1; Ar[0][1] = ca0 * a1;       Ar[0][2] = s * a1;
        Ar[1][0] = ca0 * a1;        Ar[1][1] = 1.0f - ca0 * a0; Ar[1][2] = -(s * a0);
        Ar[2][0] = -(s * a1);       Ar[2][1] = s * a0;          Ar[2][2] = 1.0f - c * x;
    }
}

// ---------------------------------------------------------------------------
// Mapping of element-frame strain rows to global dofs
// ---------------------------------------------------------------------------
// Element-frame dofs per node: u, v, w, thx, thy (the element drilling
// rotation row of T_ae is zero and carries no stiffness).
template <class R, int NN> struct GlobalMap {
    R e[3][3];      // element basis (global components)
    R t[NN][3][3];  // nodal triad vectors in global components: t[i][k] = E A_i[:,k]
    R A01[NN][2][3];// rows 0,1 of A_i
    R R2[NN][2][2]; // rotation block of T_ae
    R m[NN][2];     // drilling coupling multipliers A_i[r][2]/A_i[2][2]
    R g[NN][2];     // basis function gradients on the element basis
};

// Build the map from the double-precision frame and the triads (rounded to
// R; the products below are transformation arithmetic in the working precision).
template <class R, int NN, class E>
FS_HD void build_map(const E e[3][3], const R A[NN][3][3], const R g[NN][2], GlobalMap<R, NN> &M)
{
    for (int k = 0; k < 3; k++)
        for (int c = 0; c < 3; c++) M.e[k][c] = (R)e[k][c];
    for (int i = 0; i < NN; i++) {
        const R(&Ar)[3][3] = A[i];
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++)
                M.t[i][k][c] = Ar[0][k] * M.e[0][c] + Ar[1][k] * M.e[1][c] + Ar[2][k] * M.e[2][c];
        R inv33 = (R)1 / Ar[2][2];
        for (int r = 0; r < 2; r++) {
            for (int k = 0; k < 3; k++) M.A01[i][r][k] = Ar[r][k];
            M.m[i][r] = Ar[r][2] * inv33;
            for (int cl = 0; cl < 2; cl++) M.R2[i][r][cl] = Ar[r][cl] - inv33 * Ar[r][2] * Ar[cl][2];
        }
        M.g[i][0] = g[i][0];
        M.g[i][1] = g[i][1];
    }
}

// Expand one element-frame row c[NN][5] (u,v,w,thx,thy per node) into a row
// on the global dofs out[6*NN] (3 translations, 3 rotations per node).
template <class R, int NN>
FS_HD void expand_row(const GlobalMap<R, NN> &M, const R c[NN][5], R *out)
{
    R P0[3] = {0, 0, 0}, P1[3] = {0, 0, 0};
    for (int i = 0; i < NN; i++) {
        R mu = c[i][3] * M.m[i][0] + c[i][4] * M.m[i][1];
        for (int k = 0; k < 3; k++) {
            P0[k] += mu * M.A01[i][0][k];
            P1[k] += mu * M.A01[i][1][k];
        }
    }
    for (int j = 0; j < NN; j++) {
        R h[3];
        for (int k = 0; k < 3; k++) h[k] = (R)0.5 * (M.g[j][0] * P1[k] - M.g[j][1] * P0[k]);
        R r0 = c[j][3] * M.R2[j][0][0] + c[j][4] * M.R2[j][1][0];
        R r1 = c[j][3] * M.R2[j][0][1] + c[j][4] * M.R2[j][1][1];
        for (int q = 0; q < 3; q++) {
            out[6 * j + q] = c[j][0] * M.e[0][q] + c[j][1] * M.e[1][q] + c[j][2] * M.e[2][q] +
                             h[0] * M.t[j][0][q] + h[1] * M.t[j][1][q] + h[2] * M.t[j][2][q];
            out[6 * j + 3 + q] = r0 * M.t[j][0][q] + r1 * M.t[j][1][q];
        }
    }
}

FS_HD int lp(int r, int c) { return r * (r + 1) / 2 + c; }  // packed lower index, r >= c

// Sparse forms of expand_row for the homogeneous shells: membrane rows carry
// only in-plane translations (u, v), bending and shear rows only w and the
// rotations; materialising the dense rows would cost registers and spills.
template <class R, int NN>
FS_HD void expand_uv(const GlobalMap<R, NN> &M, const R u[NN], const R v[NN], R *out)
{
    for (int j = 0; j < NN; j++)
        for (int q = 0; q < 3; q++) {
            out[6 * j + q] = u[j] * M.e[0][q] + v[j] * M.e[1][q];
            out[6 * j + 3 + q] = 0;
        }
}

// the translations alone (3 per node): a membrane row of the compact layout
template <class R, int NN>
FS_HD void expand_uv_c(const GlobalMap<R, NN> &M, const R u[NN], const R v[NN], R *out)
{
    for (int j = 0; j < NN; j++)
        for (int q = 0; q < 3; q++) out[3 * j + q] = u[j] * M.e[0][q] + v[j] * M.e[1][q];
}

// Compact row layout of a homogeneous element (shared memory of the element
// kernel): the membrane rows keep only the translations (3 per node), the
// bending and shear rows all 6 dofs per node, the drilling row of node i only
// its 3 rotations.  Offsets in R units.
template <int NN, int NS> struct CompactRows {
    static constexpr int MS = 3 * NN;                  // membrane row length
    static constexpr int BS = 3 * MS, BSS = 6 * NN;    // bending + shear rows: start, length
    static constexpr int DR = BS + (3 + NS) * BSS;     // drilling rows: start (3 each)
    static constexpr int SIZE = DR + 3 * NN;
};

template <class R, int NN, bool HAS_W>
FS_HD void expand_wt(const GlobalMap<R, NN> &M, const R w[NN], const R tx[NN], const R ty[NN], R *out)
{
    R P0[3] = {0, 0, 0}, P1[3] = {0, 0, 0};
    for (int i = 0; i < NN; i++) {
        R mu = tx[i] * M.m[i][0] + ty[i] * M.m[i][1];
        for (int k = 0; k < 3; k++) {
            P0[k] += mu * M.A01[i][0][k];
            P1[k] += mu * M.A01[i][1][k];
        }
    }
    for (int j = 0; j < NN; j++) {
        R h[3];
        for (int k = 0; k < 3; k++) h[k] = (R)0.5 * (M.g[j][0] * P1[k] - M.g[j][1] * P0[k]);
        R r0 = tx[j] * M.R2[j][0][0] + ty[j] * M.R2[j][1][0];
        R r1 = tx[j] * M.R2[j][0][1] + ty[j] * M.R2[j][1][1];
        for (int q = 0; q < 3; q++) {
            R tv = h[0] * M.t[j][0][q] + h[1] * M.t[j][1][q] + h[2] * M.t[j][2][q];
            out[6 * j + q] = HAS_W ? w[j] * M.e[2][q] + tv : tv;
            out[6 * j + 3 + q] = r0 * M.t[j][0][q] + r1 * M.t[j][1][q];
        }
    }
}

// Per-call constant material data (host precomputed).
struct MatConst {
    double Lps[6];    // Cholesky factor of Dps, lower, packed (L00,L10,L11,L20,L21,L22)
    double Lt[3];     // Cholesky factor of (5/6) Dt, lower packed (L00,L10,L11)
    double stab_c;    // stab_fun(t,h) = t^2/(t^2 + stab_c h^2)
    double drill_scale;
    double drill_scale6;  // drill_scale / 6
    double rho;
    float Lpsf[6], Ltf[3];  // the factors rounded to float (mixed rows)
    float stab_cf;          // stab_c rounded to float
    double Dps[9];          // Dps itself (symmetrised, column-major) and (5/6) Dt:
    double Dt5[4];          // the stress resultants at the integration points
};

// entry i of a packed factor in the working precision: the float copy for
// float rows (rounded once on the host), the double factor otherwise
template <class R>
FS_HD R lpk(const double *d, const float *f, int i)
{
    if constexpr (sizeof(R) == 4) return f[i];
    return d[i];
}

// Membrane and bending rows of a homogeneous shell, mixed with the Cholesky
// factor L of Dps (rows r = 0..2: sm * sum_{c>=r} L[c][r] strain_c), written
// as global rows; returns the bending rotations for the drilling factor.
// COMPACT: membrane row r at rows + 3 NN r (translations only), bending row r
// at rows + 9 NN + 6 NN r (the CompactRows layout); otherwise rows r and 3 + r
// of stride rs.
template <class R, int NN, bool COMPACT = false>
FS_HD void homog_mb_rows(const GlobalMap<R, NN> &M, const MatConst &mc, R sm, R sb, R *rows, int rs,
                         R btx[3][NN], R bty[3][NN])
{
    for (int r = 0; r < 3; r++) {
        R c0 = r == 0 ? lpk<R>(mc.Lps, mc.Lpsf, lp(0, 0)) : (R)0;
        R c1 = r <= 1 ? lpk<R>(mc.Lps, mc.Lpsf, lp(1, r)) : (R)0;
        R c2 = lpk<R>(mc.Lps, mc.Lpsf, lp(2, r));
        R u[NN], v[NN];
        for (int j = 0; j < NN; j++) {
            u[j] = sm * (c0 * M.g[j][0] + c2 * M.g[j][1]);
            v[j] = sm * (c1 * M.g[j][1] + c2 * M.g[j][0]);
            btx[r][j] = sb * (-c1 * M.g[j][1] - c2 * M.g[j][0]);
            bty[r][j] = sb * (c0 * M.g[j][0] + c2 * M.g[j][1]);
        }
        if constexpr (COMPACT) {
            expand_uv_c<R, NN>(M, u, v, rows + 3 * NN * r);
            expand_wt<R, NN, false>(M, nullptr, btx[r], bty[r], rows + 9 * NN + 6 * NN * r);
        } else {
            expand_uv<R, NN>(M, u, v, rows + r * rs);
            expand_wt<R, NN, false>(M, nullptr, btx[r], bty[r], rows + (3 + r) * rs);
        }
    }
}

// ---------------------------------------------------------------------------
// Material factors
// ---------------------------------------------------------------------------
// Per-call constant material data (host precomputed).

// Drilling stiffness from the sum of the six nodal-basis bending diagonals:
// mean times scale, src/FEMMShellT3FFModule.jl:713-727, in double.  The FP64
// path keeps the reference's order (sum / 6 * scale); the mixed path, whose
// sum is a float, multiplies by scale / 6 (no double division).
template <class R>
FS_HD double drill_mean(double ksum, const MatConst &mc)
{
    if constexpr (sizeof(R) == 8) return ksum / 6.0 * mc.drill_scale;
    return ksum * mc.drill_scale6;
}

// Layup group (host precomputed from the laminate A,B,D,H): Cholesky factor
// of the 6x6 [A B; B D] (lower packed, 21) and of H (lower packed, 3).
struct GroupConst {
    double L6[21];
    double LH[3];
    double csmat[9];  // column-major layup csys (first column = layup reference direction)
    double thickness;
    double mass;      // mass density per unit area (laminate_inertia!)
    double moi;       // rotary inertia density
    double pad;
    float L6f[21], LHf[3];  // the factors rounded to float (mixed rows)
};


// rows_out[r] = scale * sum_{c>=r} L[c][r] rows_in[c]   (L^T applied to stacked rows)
template <class R, int NN, int NR>
FS_HD void mix_rows(const double *Lpk, const float *Lpkf, R scale, const R in[NR][NN][5], R out[NR][NN][5])
{
    for (int r = 0; r < NR; r++) {
        R f[NR];
        for (int c = 0; c < NR; c++) f[c] = (c >= r) ? scale * lpk<R>(Lpk, Lpkf, lp(c, r)) : (R)0;
        for (int i = 0; i < NN; i++)
            for (int q = 0; q < 5; q++) {
                R s = 0;
                for (int c = r; c < NR; c++) s += f[c] * in[c][i][q];
                out[r][i][q] = s;
            }
    }
}

// Layup-to-element angle (reference Layup2ElementAngle, src/TransformerModule.jl:92-105)
FS_HD void layup_angle(const double e[3][3], const double cs[9], double &m, double &n)
{
    // M = E^T csmat, 2x2 leading block, columns normalised
    double a11 = e[0][0] * cs[0] + e[0][1] * cs[1] + e[0][2] * cs[2];
    double a21 = e[1][0] * cs[0] + e[1][1] * cs[1] + e[1][2] * cs[2];
    double a12 = e[0][0] * cs[3] + e[0][1] * cs[4] + e[0][2] * cs[5];
    double a22 = e[1][0] * cs[3] + e[1][1] * cs[4] + e[1][2] * cs[5];
    double n1 = sqrt(a11 * a11 + a21 * a21), n2 = sqrt(a12 * a12 + a22 * a22);
    a11 /= n1; a21 /= n1; a12 /= n2; a22 /= n2;
    m = (a11 + a22) / 2.0;
    double nn = (a12 - a21) / 2.0;
    double q = 1.0 - m * m;
    n = (nn >= 0.0 ? 1.0 : -1.0) * sqrt(q > 0.0 ? q : 0.0);
}

// Rotate the membrane and bending element-frame rows by Tbar and the shear
// rows by Tts (plane_stress_Tbar_matrix!, src/CompositeLayupModule.jl:364-378;
// transverse_shear_T_matrix!, :463-471): strain' = T strain.
template <class R, int NN>
FS_HD void rotate3(double m, double n, R rows[3][NN][5])
{
    double T[3][3] = {{m * m, n * n, -(m * n)}, {n * n, m * m, (m * n)}, {2 * (m * n), -2 * (m * n), m * m - n * n}};
    for (int i = 0; i < NN; i++)
        for (int q = 0; q < 5; q++) {
            R a = rows[0][i][q], b = rows[1][i][q], c = rows[2][i][q];
            rows[0][i][q] = (R)T[0][0] * a + (R)T[0][1] * b + (R)T[0][2] * c;
            rows[1][i][q] = (R)T[1][0] * a + (R)T[1][1] * b + (R)T[1][2] * c;
            rows[2][i][q] = (R)T[2][0] * a + (R)T[2][1] * b + (R)T[2][2] * c;
        }
}
template <class R, int NN>
FS_HD void rotate2(double m, double n, R rows[2][NN][5])
{
    for (int i = 0; i < NN; i++)
        for (int q = 0; q < 5; q++) {
            R a = rows[0][i][q], b = rows[1][i][q];
            rows[0][i][q] = (R)m * a - (R)n * b;
            rows[1][i][q] = (R)n * a + (R)m * b;
        }
}

// ---------------------------------------------------------------------------
// Element inputs
// ---------------------------------------------------------------------------
template <int NN> struct ElemIn {
    double X[NN][3];     // node coordinates
    double nrm[NN][3];   // nodal normals
    float nrmf[NN][3];   // the same rounded to float (the float rows' triads)
    bool valid[NN];      // normal valid flags
    double t;            // thickness
    int group;           // layup group (composite)
};

// ---------------------------------------------------------------------------
// T3FF: rows of one element
// ---------------------------------------------------------------------------
// Number of Gram rows: membrane+bending 6, shear 2 (average B) or 6
// (average K), drilling 3.
template <bool AVGK> struct T3Rows { static const int NS = AVGK ? 6 : 2; static const int N = 6 + NS + 3; };

// T3 element-frame shear rows for the node ordering (s,p,q)
// (reference _add_Bsmat_o!, src/FEMMShellT3FFModule.jl:486-526).
template <class R>
FS_HD void t3_bs_ordering(const R x[3], const R y[3], R Ae, int s, int p, int q, R Bs[2][3][5], R w)
{
    R a = x[p] - x[s], b = y[p] - y[s], c = x[q] - x[s], d = y[q] - y[s];
    R mm = w / (2 * Ae);
    Bs[0][s][2] += mm * (b - d);  Bs[1][s][2] += mm * (c - a);
    Bs[0][s][4] += mm * Ae;       Bs[1][s][3] += -mm * Ae;
    Bs[0][p][2] += mm * d;        Bs[1][p][2] += -mm * c;
    Bs[0][p][3] += -mm * b * d / 2; Bs[1][p][3] += mm * b * c / 2;
    Bs[0][p][4] += mm * a * d / 2;  Bs[1][p][4] += -mm * a * c / 2;
    Bs[0][q][2] += -mm * b;       Bs[1][q][2] += mm * a;
    Bs[0][q][3] += mm * b * d / 2;  Bs[1][q][3] += -mm * a * d / 2;
    Bs[0][q][4] += -mm * b * c / 2; Bs[1][q][4] += mm * a * c / 2;
}

// Computes the Gram rows (global dofs, 18 wide) of one T3FF / T3FFComp
// element.  Returns 0 on success.  `rows` is written with row stride `rs`,
// or (COMPACT, homogeneous elements) in the CompactRows<3, NS> layout.
template <class R, bool COMP, bool AVGK, bool COMPACT = false>
FS_HD int t3_rows(const ElemIn<3> &in, const MatConst &mc, const GroupConst *gc, R *rows, int rs)
{
    static_assert(!(COMP && COMPACT), "the compact layout is for homogeneous elements");
    // --- frame and element coordinates (double) ---
    double J0[3], J1[3], e[3][3];
    for (int c = 0; c < 3; c++) {
        J0[c] = in.X[1][c] - in.X[0][c];
        J1[c] = in.X[2][c] - in.X[0][c];
    }
    make_frame(J0, J1, e);
    const double t = COMP ? gc->thickness : in.t;
    // element coordinates x, y of the nodes, basis gradients, area and the
    // stabilisation factor t^2 / (t^2 + c h^2), h^2 = 2 Ae
    R g[3][2], x[3], y[3], AeR, stab;
    if constexpr (sizeof(R) == 8) {
        double a = dot3(J0, e[0]), b = dot3(J0, e[1]);
        double cc = dot3(J1, e[0]), d = dot3(J1, e[1]);
        double Jd = a * d - b * cc;
        double Ae = Jd / 2;
        double iJ = 1.0 / Jd;
        g[0][0] = (b - d) * iJ; g[1][0] = d * iJ; g[2][0] = -b * iJ;
        g[0][1] = (cc - a) * iJ; g[1][1] = -cc * iJ; g[2][1] = a * iJ;
        x[0] = 0; x[1] = a; x[2] = cc;
        y[0] = 0; y[1] = b; y[2] = d;
        AeR = Ae;
        double h2 = 2 * Ae;
        stab = t * t / (t * t + mc.stab_c * h2);
    } else {
        // coordinates and the differences of the gradients in double (the
        // differences of nearby coordinates lose digits in float), rounded
        // once; the rest in float
        const double a = dot3(J0, e[0]), b = dot3(J0, e[1]);
        const double cc = dot3(J1, e[0]), d = dot3(J1, e[1]);
        const double Jd = a * d - b * cc;
        const float iJ = 1.0f / (float)Jd;
        g[0][0] = (float)(b - d) * iJ; g[1][0] = (float)d * iJ; g[2][0] = -(float)b * iJ;
        g[0][1] = (float)(cc - a) * iJ; g[1][1] = -(float)cc * iJ; g[2][1] = (float)a * iJ;
        x[0] = 0; x[1] = (float)a; x[2] = (float)cc;
        y[0] = 0; y[1] = (float)b; y[2] = (float)d;
        AeR = (float)(Jd / 2);
        const float tf = (float)t;
        stab = tf * tf / (tf * tf + mc.stab_cf * (2 * AeR));
    }
    // --- triads ---
    R A[3][3][3];
    GlobalMap<R, 3> M;
    if constexpr (sizeof(R) == 4) {
        float ef[3][3];
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) ef[k][c] = (float)e[k][c];
        for (int i = 0; i < 3; i++) nodal_triad_f(ef, in.nrmf[i], in.valid[i], A[i]);
        build_map<R, 3>(ef, A, g, M);
    } else {
        for (int i = 0; i < 3; i++) nodal_triad_r<R>(e, in.nrm[i], in.valid[i], A[i]);
        build_map<R, 3>(e, A, g, M);
    }

    constexpr int NS = T3Rows<AVGK>::NS;
    // --- transverse shear rows in the element frame (w, thx, thy per node) ---
    R sh[NS][3][5];
    for (int r = 0; r < NS; r++)
        for (int i = 0; i < 3; i++)
            for (int q = 0; q < 5; q++) sh[r][i][q] = 0;
    if (AVGK) {
        t3_bs_ordering<R>(x, y, AeR, 0, 1, 2, (R(*)[3][5])sh[0], (R)1);
        t3_bs_ordering<R>(x, y, AeR, 1, 2, 0, (R(*)[3][5])sh[2], (R)1);
        t3_bs_ordering<R>(x, y, AeR, 2, 0, 1, (R(*)[3][5])sh[4], (R)1);
    } else {
        t3_bs_ordering<R>(x, y, AeR, 0, 1, 2, (R(*)[3][5])sh[0], (R)(1.0 / 3));
        t3_bs_ordering<R>(x, y, AeR, 1, 2, 0, (R(*)[3][5])sh[0], (R)(1.0 / 3));
        t3_bs_ordering<R>(x, y, AeR, 2, 0, 1, (R(*)[3][5])sh[0], (R)(1.0 / 3));
    }
    // rotations of every bending/shear row, for the drilling factor
    R rtx[3 + NS][3], rty[3 + NS][3];
    if constexpr (!COMP) {
        // --- homogeneous: sparse rows, Dps and (5/6)Dt Cholesky mixing ---
        R tr_ = (R)t;
        homog_mb_rows<R, 3, COMPACT>(M, mc, sqrt(tr_ * AeR), sqrt(tr_ * tr_ * tr_ / 12 * AeR), rows, rs,
                                     (R(*)[3])rtx[0], (R(*)[3])rty[0]);
        R ws = sqrt(tr_ * stab * AeR * (R)(AVGK ? 1.0 / 3 : 1.0));
        R l00 = lpk<R>(mc.Lt, mc.Ltf, lp(0, 0)), l10 = lpk<R>(mc.Lt, mc.Ltf, lp(1, 0)), l11 = lpk<R>(mc.Lt, mc.Ltf, lp(1, 1));
        for (int o = 0; o < NS / 2; o++)
            for (int r = 0; r < 2; r++) {
                R f0 = r == 0 ? ws * l00 : (R)0, f1 = ws * (r == 0 ? l10 : l11);
                R w[3];
                for (int i = 0; i < 3; i++) {
                    w[i] = f0 * sh[2 * o][i][2] + f1 * sh[2 * o + 1][i][2];
                    rtx[3 + 2 * o + r][i] = f0 * sh[2 * o][i][3] + f1 * sh[2 * o + 1][i][3];
                    rty[3 + 2 * o + r][i] = f0 * sh[2 * o][i][4] + f1 * sh[2 * o + 1][i][4];
                }
                R *row = COMPACT ? rows + CompactRows<3, NS>::BS + CompactRows<3, NS>::BSS * (3 + 2 * o + r)
                                 : rows + (6 + 2 * o + r) * rs;
                expand_wt<R, 3, true>(M, w, rtx[3 + 2 * o + r], rty[3 + 2 * o + r], row);
            }
    } else {
        // --- layered: membrane and bending rows rotated by the layup angle and
        //     mixed with the 6x6 [A B; B D] factor, shear with H ---
        R mb[6][3][5];
        for (int r = 0; r < 6; r++)
            for (int i = 0; i < 3; i++)
                for (int q = 0; q < 5; q++) mb[r][i][q] = 0;
        for (int i = 0; i < 3; i++) {
            mb[0][i][0] = g[i][0];
            mb[1][i][1] = g[i][1];
            mb[2][i][0] = g[i][1]; mb[2][i][1] = g[i][0];
            mb[3][i][4] = g[i][0];
            mb[4][i][3] = -g[i][1];
            mb[5][i][3] = -g[i][0]; mb[5][i][4] = g[i][1];
        }
        R mixed[6 + NS][3][5];
        double lm, ln;
        layup_angle(e, gc->csmat, lm, ln);
        rotate3<R, 3>(lm, ln, (R(*)[3][5])mb[0]);
        rotate3<R, 3>(lm, ln, (R(*)[3][5])mb[3]);
        mix_rows<R, 3, 6>(gc->L6, gc->L6f, sqrt(AeR), mb, (R(*)[3][5])mixed[0]);
        R ws = stab * AeR * (R)(AVGK ? 1.0 / 3 : 1.0);
        for (int o = 0; o < NS / 2; o++) {
            rotate2<R, 3>(lm, ln, (R(*)[3][5])sh[2 * o]);
            mix_rows<R, 3, 2>(gc->LH, gc->LHf, sqrt(ws), (R(*)[3][5])sh[2 * o], (R(*)[3][5])mixed[6 + 2 * o]);
        }
        for (int r = 0; r < 6 + NS; r++) expand_row<R, 3>(M, (const R(*)[5])mixed[r], rows + r * rs);
        // drilling factor: every mixed row may carry rotations here
        R ksumr = 0;
        for (int i = 0; i < 3; i++)
            for (int cl = 0; cl < 2; cl++)
                for (int r = 0; r < 6 + NS; r++) {
                    R v = mixed[r][i][3] * M.R2[i][0][cl] + mixed[r][i][4] * M.R2[i][1][cl];
                    ksumr += v * v;
                }
        double kavg = drill_mean<R>((double)ksumr, mc);
        R sk = kavg > 0.0 ? sqrt((R)kavg) : (R)0;
        for (int i = 0; i < 3; i++) {
            R *o = rows + (6 + NS + i) * rs;
            for (int q = 0; q < 18; q++) o[q] = 0;
            if (in.valid[i])
                for (int c = 0; c < 3; c++) o[6 * i + 3 + c] = sk * M.t[i][2][c];
        }
        return (kavg < 0.0) ? 2 : 0;
    }
    // --- drilling factor: mean of the nodal-basis bending diagonals,
    //     src/FEMMShellT3FFModule.jl:713-727 (mean and scale in double) ---
    R ksumr = 0;
    for (int i = 0; i < 3; i++)
        for (int cl = 0; cl < 2; cl++)
            for (int r = 0; r < 3 + NS; r++) {
                R v = rtx[r][i] * M.R2[i][0][cl] + rty[r][i] * M.R2[i][1][cl];
                ksumr += v * v;
            }
    double kavg = drill_mean<R>((double)ksumr, mc);
    R sk = kavg > 0.0 ? sqrt((R)kavg) : (R)0;
    for (int i = 0; i < 3; i++) {
        if constexpr (COMPACT) {
            R *o = rows + CompactRows<3, NS>::DR + 3 * i;
            for (int c = 0; c < 3; c++) o[c] = in.valid[i] ? sk * M.t[i][2][c] : (R)0;
        } else {
            R *o = rows + (6 + NS + i) * rs;
            for (int q = 0; q < 18; q++) o[q] = 0;
            if (in.valid[i])
                for (int c = 0; c < 3; c++) o[6 * i + 3 + c] = sk * M.t[i][2][c];
        }
    }
    return (kavg < 0.0) ? 2 : 0;
}

// ---------------------------------------------------------------------------
// Q4RS: rows of one quadrature point
// ---------------------------------------------------------------------------
static constexpr double Q4_GP = 0.577350269189626;  // FinEtools GaussRule(2,2) abscissa

FS_HD void q4_point(int j, double &xi, double &eta)
{
    xi = (j < 2 ? -Q4_GP : Q4_GP);
    eta = ((j & 1) ? Q4_GP : -Q4_GP);
}

template <class T>
FS_HD void q4_dbasis_t(T xi, T eta, T gp[4][2])
{
    const T q = (T)0.25, one = (T)1;
    gp[0][0] = -q * (one - eta); gp[0][1] = -q * (one - xi);
    gp[1][0] = q * (one - eta);  gp[1][1] = -q * (one + xi);
    gp[2][0] = q * (one + eta);  gp[2][1] = q * (one + xi);
    gp[3][0] = -q * (one + eta); gp[3][1] = q * (one - xi);
}

FS_HD void q4_dbasis(double xi, double eta, double gp[4][2])
{
    gp[0][0] = -0.25 * (1 - eta); gp[0][1] = -0.25 * (1 - xi);
    gp[1][0] = 0.25 * (1 - eta);  gp[1][1] = -0.25 * (1 + xi);
    gp[2][0] = 0.25 * (1 + eta);  gp[2][1] = 0.25 * (1 + xi);
    gp[3][0] = -0.25 * (1 + eta); gp[3][1] = 0.25 * (1 - xi);
}

// q4_dbasis at Gauss point j (q4_point) from the two products it can take,
// 0.25 (1 -+ 0.5773...) evaluated at compile time: the same values, chosen
// by the signs of xi and eta instead of computed.
FS_HD void q4_dbasis_gp(int j, double gp[4][2])
{
    constexpr double QA = 0.25 * (1.0 - Q4_GP), QB = 0.25 * (1.0 + Q4_GP);
    const bool xp = j >= 2, ep = (j & 1) != 0;  // xi > 0, eta > 0
    const double e1m = ep ? QA : QB, e1p = ep ? QB : QA;  // 0.25 (1 - eta), 0.25 (1 + eta)
    const double x1m = xp ? QA : QB, x1p = xp ? QB : QA;  // 0.25 (1 - xi), 0.25 (1 + xi)
    gp[0][0] = -e1m; gp[0][1] = -x1m;
    gp[1][0] = e1m;  gp[1][1] = -x1p;
    gp[2][0] = e1p;  gp[2][1] = x1p;
    gp[3][0] = -e1p; gp[3][1] = x1m;
}

// MITC transverse shear rows in the element frame
// (reference _Bsmat, src/FEMMShellQ4RSModule.jl:702-751), regrouped: each
// entry is p*LA*fa(node) + q*LB*fb(node) with (p,q) = (sa,sb) for gxz and
// (-ca,-cb) for gyz.
template <class R>
FS_HD void q4_bs(const R X[4], const R Y[4], R r, R s, R Bs[2][4][5])
{
    R J11 = (X[0] * (s - 1) - X[1] * (s - 1) + X[2] * (s + 1) - X[3] * (s + 1)) / 4;
    R J21 = (Y[0] * (s - 1) - Y[1] * (s - 1) + Y[2] * (s + 1) - Y[3] * (s + 1)) / 4;
    R J12 = (X[0] * (r - 1) - X[1] * (r + 1) + X[2] * (r + 1) - X[3] * (r - 1)) / 4;
    R J22 = (Y[0] * (r - 1) - Y[1] * (r + 1) + Y[2] * (r + 1) - Y[3] * (r - 1)) / 4;
    R A = sqrt(J11 * J11 + J21 * J21), B = sqrt(J12 * J12 + J22 * J22);
    R ca = J11 / A, sa = J21 / A, cb = J12 / B, sb = J22 / B;
    R detJ = J11 * J22 - J12 * J21;
    R Ax = X[0] - X[1] - X[2] + X[3], Ay = Y[0] - Y[1] - Y[2] + Y[3];
    R Bx = X[0] - X[1] + X[2] - X[3], By = Y[0] - Y[1] + Y[2] - Y[3];
    R Cx = X[0] + X[1] - X[2] - X[3], Cy = Y[0] + Y[1] - Y[2] - Y[3];
    R LA = sqrt((Ax + Bx * s) * (Ax + Bx * s) + (Ay + By * s) * (Ay + By * s));
    R LB = sqrt((Bx * r + Cx) * (Bx * r + Cx) + (By * r + Cy) * (By * r + Cy));
    R rp = r + 1, rm = r - 1, sp = s + 1, sm = s - 1;
    R d16 = 1 / (16 * detJ), d32 = 1 / (32 * detJ);
    // node-wise factors of the LA (tying along r) and LB (along s) terms
    R fw_a[4] = {rp, -rm, rm, -rp}, fw_b[4] = {-sp, sp, -sm, sm};
    R fx_a[4] = {-(Y[0] - Y[3]) * rp, (Y[1] - Y[2]) * rm, (Y[1] - Y[2]) * rm, -(Y[0] - Y[3]) * rp};
    R fx_b[4] = {(Y[0] - Y[1]) * sp, (Y[0] - Y[1]) * sp, (Y[2] - Y[3]) * sm, (Y[2] - Y[3]) * sm};
    R fy_a[4] = {(X[0] - X[3]) * rp, -(X[1] - X[2]) * rm, -(X[1] - X[2]) * rm, (X[0] - X[3]) * rp};
    R fy_b[4] = {-(X[0] - X[1]) * sp, -(X[0] - X[1]) * sp, -(X[2] - X[3]) * sm, -(X[2] - X[3]) * sm};
    for (int row = 0; row < 2; row++) {
        R pa = (row == 0 ? sa : -ca) * LA, qb = (row == 0 ? sb : -cb) * LB;
        for (int k = 0; k < 4; k++) {
            Bs[row][k][0] = 0;
            Bs[row][k][1] = 0;
            Bs[row][k][2] = (pa * fw_a[k] + qb * fw_b[k]) * d16;
            Bs[row][k][3] = (pa * fx_a[k] + qb * fx_b[k]) * d32;
            Bs[row][k][4] = (pa * fy_a[k] + qb * fy_b[k]) * d32;
        }
    }
}

// Q4 element-level constants shared by the four quadrature points.
struct Q4Elem {
    double Xr[4][3];   // node coordinates relative to the centroid
    float Xf[4][3];    // the same rounded to float (the float rows' element coordinates)
    double stab;       // shear stabilisation t^2 / (t^2 + c h^2), h = max distance from node 1
};

// `t` is the element (or layup) thickness, `stab_c` the stabilisation constant.
FS_HD void q4_prepare(const ElemIn<4> &in, double t, double stab_c, Q4Elem &qe)
{
    double cen[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++)
        for (int c = 0; c < 3; c++) cen[c] += in.X[a][c];
    for (int c = 0; c < 3; c++) cen[c] /= 4;
    double mx = 0.0;
    for (int a = 0; a < 4; a++) {
        for (int c = 0; c < 3; c++) {
            qe.Xr[a][c] = in.X[a][c] - cen[c];
            qe.Xf[a][c] = (float)qe.Xr[a][c];
        }
        if (a > 0) {
            double dx = in.X[a][0] - in.X[0][0], dy = in.X[a][1] - in.X[0][1], dz = in.X[a][2] - in.X[0][2];
            double dd = dx * dx + dy * dy + dz * dz;
            mx = dd > mx ? dd : mx;
        }
    }
    qe.stab = t * t / (t * t + stab_c * mx);
}

// Compact rows of one quadrature point of a homogeneous Q4 element (shared
// memory of the element kernel): the 3 membrane rows keep the translations
// only (12 values), the 3 bending and 2 shear rows all 24 dofs.  Offsets in
// R units; the element's 4 drilling rows (3 rotations each) follow the four
// points' blocks.
struct Q4Compact {
    static constexpr int MS = 12;          // membrane row length
    static constexpr int BS = 36, BSS = 24; // bending + shear rows: start, length
    static constexpr int GP = BS + 5 * BSS; // one point's block (156)
    static constexpr int DR = 4 * GP;       // drilling rows: start (3 each)
    static constexpr int SIZE = DR + 12;    // 636
};

// Rows of quadrature point j (8 rows: membrane+bending 6, shear 2) on the
// global dofs (24 wide), plus this point's contribution to the drilling
// traces tr(P K_rr P) of each node (src/FEMMShellQ4RSModule.jl:807-838).
// Returns nonzero on a singular metric (src/FEMMShellQ4RSModule.jl:308-311).
// COMPACT (homogeneous elements): `rows` is the point's Q4Compact block and
// `rs` is not used.
template <class R, bool COMP, bool COMPACT = false, bool FFRAME = false>
FS_HD int q4_point_rows(const ElemIn<4> &in, const Q4Elem &qe, int j, const MatConst &mc,
                        const GroupConst *gc, R *rows, int rs, double trace[4])
{
    static_assert(!(COMP && COMPACT), "the compact layout is for homogeneous elements");
    static_assert(!FFRAME || sizeof(R) == 4, "the float frame is for float rows");
    double xi, eta, gp[4][2];
    q4_point(j, xi, eta);
    q4_dbasis_gp(j, gp);
    // basis gradients in the working precision (float rows: evaluated in float)
    R gq[4][2], xir, etar;
    if constexpr (sizeof(R) == 4) {
        xir = j < 2 ? -(float)Q4_GP : (float)Q4_GP;
        etar = (j & 1) ? (float)Q4_GP : -(float)Q4_GP;
        q4_dbasis_t<R>(xir, etar, gq);
    } else {
        xir = xi;
        etar = eta;
        for (int a = 0; a < 4; a++) {
            gq[a][0] = gp[a][0];
            gq[a][1] = gp[a][1];
        }
    }
    // tangents and frame: in double from the centroid-relative coordinates,
    // rounded once to the working precision (tangents summed in float from
    // rounded coordinates lose about one more digit); or (FFRAME, FS_MIXED's
    // cheaper choice) in float from the float coordinates and gradients, off
    // the FP64 pipe
    R J0r[3], J1r[3], eR[3][3];
    double e[3][3];  // the double frame (FFRAME: the float one widened, for the layup angle)
    if constexpr (FFRAME) {
        for (int c = 0; c < 3; c++) {
            J0r[c] = qe.Xf[0][c] * gq[0][0] + qe.Xf[1][c] * gq[1][0] + qe.Xf[2][c] * gq[2][0] + qe.Xf[3][c] * gq[3][0];
            J1r[c] = qe.Xf[0][c] * gq[0][1] + qe.Xf[1][c] * gq[1][1] + qe.Xf[2][c] * gq[2][1] + qe.Xf[3][c] * gq[3][1];
        }
        make_frame_f(J0r, J1r, eR);
        if constexpr (COMP)
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) e[k][c] = eR[k][c];
    } else {
        double J0[3], J1[3];
        for (int c = 0; c < 3; c++) {
            J0[c] = qe.Xr[0][c] * gp[0][0] + qe.Xr[1][c] * gp[1][0] + qe.Xr[2][c] * gp[2][0] + qe.Xr[3][c] * gp[3][0];
            J1[c] = qe.Xr[0][c] * gp[0][1] + qe.Xr[1][c] * gp[1][1] + qe.Xr[2][c] * gp[2][1] + qe.Xr[3][c] * gp[3][1];
        }
        make_frame(J0, J1, e);
        for (int c = 0; c < 3; c++) {
            J0r[c] = (R)J0[c];
            J1r[c] = (R)J1[c];
        }
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) eR[k][c] = (R)e[k][c];
    }
    // element coordinates (centroid relative)
    R X[4], Y[4];
    for (int a = 0; a < 4; a++) {
        R xr[3];
        for (int c = 0; c < 3; c++) xr[c] = sizeof(R) == 4 ? (R)qe.Xf[a][c] : (R)qe.Xr[a][c];
        X[a] = dot3(xr, eR[0]);
        Y[a] = dot3(xr, eR[1]);
    }
    // surface Jacobian |J0 x J1| in the working precision
    R Jac;
    {
        R nJ[3];
        cross3(J0r, J1r, nJ);
        Jac = sqrt(dot3(nJ, nJ));
    }
    R G11 = dot3(J0r, J0r), G12 = dot3(J0r, J1r), G22 = dot3(J1r, J1r);
    R detG = G11 * G22 - G12 * G12;
    if (detG == (R)0) return 4;
    R i11 = G22 / detG, i12 = -G12 / detG, i22 = G11 / detG;
    R g[4][2];
    // g_a = J invG gradNparams_a, projected on e1, e2
    R pj0[2] = {dot3(eR[0], J0r), dot3(eR[1], J0r)}, pj1[2] = {dot3(eR[0], J1r), dot3(eR[1], J1r)};
    for (int a = 0; a < 4; a++) {
        R t1 = i11 * gq[a][0] + i12 * gq[a][1];
        R t2 = i12 * gq[a][0] + i22 * gq[a][1];
        g[a][0] = pj0[0] * t1 + pj1[0] * t2;
        g[a][1] = pj0[1] * t1 + pj1[1] * t2;
    }
    R A[4][3][3];
    GlobalMap<R, 4> M;
    if constexpr (sizeof(R) == 4) {
        for (int i = 0; i < 4; i++) nodal_triad_f(eR, in.nrmf[i], in.valid[i], A[i]);
        build_map<R, 4>(eR, A, g, M);
    } else {
        for (int i = 0; i < 4; i++) nodal_triad_r<R>(e, in.nrm[i], in.valid[i], A[i]);
        build_map<R, 4>(e, A, g, M);
    }
    R sh[2][4][5];
    q4_bs<R>(X, Y, xir, etar, sh);
    const R stab = (R)qe.stab;
    if constexpr (!COMP) {
        R tr_ = (R)in.t, jr = Jac;
        R btx[3][4], bty[3][4];
        homog_mb_rows<R, 4, COMPACT>(M, mc, sqrt(tr_ * jr), sqrt(tr_ * tr_ * tr_ / 12 * jr), rows, rs, btx, bty);
        R ws = sqrt(tr_ * stab * jr);
        R l00 = lpk<R>(mc.Lt, mc.Ltf, lp(0, 0)), l10 = lpk<R>(mc.Lt, mc.Ltf, lp(1, 0)), l11 = lpk<R>(mc.Lt, mc.Ltf, lp(1, 1));
        for (int r = 0; r < 2; r++) {
            R f0 = r == 0 ? ws * l00 : (R)0, f1 = ws * (r == 0 ? l10 : l11);
            R w[4], tx[4], ty[4];
            for (int i = 0; i < 4; i++) {
                w[i] = f0 * sh[0][i][2] + f1 * sh[1][i][2];
                tx[i] = f0 * sh[0][i][3] + f1 * sh[1][i][3];
                ty[i] = f0 * sh[0][i][4] + f1 * sh[1][i][4];
            }
            expand_wt<R, 4, true>(M, w, tx, ty,
                                  COMPACT ? rows + Q4Compact::BS + Q4Compact::BSS * (3 + r) : rows + (6 + r) * rs);
        }
    } else {
        R mb[6][4][5];
        for (int r = 0; r < 6; r++)
            for (int i = 0; i < 4; i++)
                for (int q = 0; q < 5; q++) mb[r][i][q] = 0;
        for (int i = 0; i < 4; i++) {
            mb[0][i][0] = g[i][0];
            mb[1][i][1] = g[i][1];
            mb[2][i][0] = g[i][1]; mb[2][i][1] = g[i][0];
            mb[3][i][4] = g[i][0];
            mb[4][i][3] = -g[i][1];
            mb[5][i][3] = -g[i][0]; mb[5][i][4] = g[i][1];
        }
        R mixed[8][4][5];
        double lm, ln;
        layup_angle(e, gc->csmat, lm, ln);
        rotate3<R, 4>(lm, ln, (R(*)[4][5])mb[0]);
        rotate3<R, 4>(lm, ln, (R(*)[4][5])mb[3]);
        mix_rows<R, 4, 6>(gc->L6, gc->L6f, sqrt(Jac), mb, (R(*)[4][5])mixed[0]);
        rotate2<R, 4>(lm, ln, sh);
        mix_rows<R, 4, 2>(gc->LH, gc->LHf, sqrt(stab * Jac), sh, (R(*)[4][5])mixed[6]);
        for (int r = 0; r < 8; r++) expand_row<R, 4>(M, (const R(*)[5])mixed[r], rows + r * rs);
    }
    // drilling traces: sum over rows of |b|^2 - (b.n)^2 on the rotation block
    // (float rows: the float copy of the normals, the same values as the
    // double normals rounded here)
    for (int k = 0; k < 4; k++) {
        R nv[3];
        for (int c = 0; c < 3; c++) nv[c] = sizeof(R) == 4 ? (R)in.nrmf[k][c] : (R)in.nrm[k][c];
        R nn = sqrt(dot3(nv, nv));
        R u[3] = {0, 0, 0};
        if (nn > (R)0) { u[0] = nv[0] / nn; u[1] = nv[1] / nn; u[2] = nv[2] / nn; }
        R tr = 0;
        // compact: the membrane rows have no rotations (their terms are zero)
        for (int r = COMPACT ? 3 : 0; r < 8; r++) {
            const R *o = (COMPACT ? rows + Q4Compact::BS + Q4Compact::BSS * (r - 3) : rows + r * rs) + 6 * k + 3;
            R bn = o[0] * u[0] + o[1] * u[1] + o[2] * u[2];
            tr += o[0] * o[0] + o[1] * o[1] + o[2] * o[2] - bn * bn;
        }
        trace[k] = (double)tr;
    }
    return 0;
}

// Drilling rows of a Q4 element from the summed traces
// (src/FEMMShellQ4RSModule.jl:807-859): kavg = scale * mean over nodes with
// a valid nonzero normal of max(0, tr/2); row k = sqrt(kavg) n_k on the
// rotations of node k.
template <class R>
FS_HD void q4_drill_rows(const ElemIn<4> &in, const double trace[4], double scale, R *rows, int rs)
{
    double sum = 0.0;
    int cnt = 0;
    bool use[4];
    for (int k = 0; k < 4; k++) {
        const double *nv = in.nrm[k];
        use[k] = in.valid[k] && (sqrt(dot3(nv, nv)) != 0.0);
        if (use[k]) {
            double v = trace[k] / 2.0;
            sum += v > 0.0 ? v : 0.0;
            cnt++;
        }
    }
    double kavg = (cnt ? sum / cnt : 0.0) * scale;
    double sk = kavg > 0.0 ? sqrt(kavg) : 0.0;
    for (int k = 0; k < 4; k++) {
        R *o = rows + k * rs;
        for (int q = 0; q < 24; q++) o[q] = 0;
        if (use[k] && kavg != 0.0)
            for (int c = 0; c < 3; c++) o[6 * k + 3 + c] = (R)(sk * in.nrm[k][c]);
    }
}

// q4_drill_rows in float (FS_MIXED's float frames): float traces and normals
FS_HD void q4_drill_rows_f(const ElemIn<4> &in, const float trace[4], float scale, float *rows, int rs)
{
    float sum = 0.f;
    int cnt = 0;
    bool use[4];
    for (int k = 0; k < 4; k++) {
        const float *nv = in.nrmf[k];
        use[k] = in.valid[k] && (dot3(nv, nv) != 0.f);
        if (use[k]) {
            const float v = trace[k] * 0.5f;
            sum += v > 0.f ? v : 0.f;
            cnt++;
        }
    }
    const float kavg = (cnt ? sum / (float)cnt : 0.f) * scale;
    const float sk = kavg > 0.f ? sqrtf(kavg) : 0.f;
    for (int k = 0; k < 4; k++) {
        float *o = rows + k * rs;
        for (int q = 0; q < 24; q++) o[q] = 0;
        if (use[k] && kavg != 0.f)
            for (int c = 0; c < 3; c++) o[6 * k + 3 + c] = sk * in.nrmf[k][c];
    }
}

// ---------------------------------------------------------------------------
// Lumped mass (src/FEMMShellT3FFModule.jl:770-787, src/FEMMShellQ4RSModule.jl:981-997
// and the layered variants)
// ---------------------------------------------------------------------------
template <int NN>
FS_HD void lumped_mass(const ElemIn<NN> &in, double rho, bool comp, const GroupConst *gc, double &tm, double &rm)
{
    double t = comp ? gc->thickness : in.t;
    if (NN == 3) {
        double J0[3], J1[3], e[3][3];
        for (int c = 0; c < 3; c++) {
            J0[c] = in.X[1][c] - in.X[0][c];
            J1[c] = in.X[2][c] - in.X[0][c];
        }
        make_frame(J0, J1, e);
        double a = dot3(J0, e[0]), b = dot3(J0, e[1]), c = dot3(J1, e[0]), d = dot3(J1, e[1]);
        double Ae = (a * d - b * c) / 2;
        if (comp) {
            tm = gc->mass * (Ae / 3);
            rm = gc->moi * (Ae / 3);
        } else {
            tm = rho * (t * Ae) / 3;
            rm = rho * (t * t * t / 12 * Ae) / 3;
        }
    } else {
        double ts = 0.0, rs = 0.0;
        for (int j = 0; j < 4; j++) {
            double xi, eta, gp[4][2];
            q4_point(j, xi, eta);
            q4_dbasis(xi, eta, gp);
            double J0[3] = {0, 0, 0}, J1[3] = {0, 0, 0};
            for (int a = 0; a < 4; a++)
                for (int c = 0; c < 3; c++) {
                    J0[c] += in.X[a][c] * gp[a][0];
                    J1[c] += in.X[a][c] * gp[a][1];
                }
            double nJ[3];
            cross3(J0, J1, nJ);
            double Jac = sqrt(dot3(nJ, nJ));
            if (comp) {
                ts += gc->mass * Jac;
                rs += gc->moi * Jac;
            } else {
                ts += rho * t * Jac;
                rs += rho * t * t * t / 12 * Jac;
            }
        }
        tm = ts / 4;
        rm = rs / 4;
    }
}

// ---------------------------------------------------------------------------
// Stress resultants at the integration points of the homogeneous shells
// (inspectintegpoints, src/FEMMShellT3FFModule.jl:850-962: the centroid of a
// T3FF element; src/FEMMShellQ4RSModule.jl:1061-1170: the Gauss points of a
// Q4RS element).  The element-frame strain rows (membrane, curvature or
// transverse shear) are expanded to the global dofs with the map of the
// stiffness rows -- the same T_ae T_ga the reference applies to the element
// displacements -- and applied to them; the resultant (t Dps strain, t^3/12
// Dps curvature, t stab (5/6) Dt shear) is seen in the output csys by the
// angle of Layup2ElementAngle(E_G, csmat).  Double precision throughout.
// ---------------------------------------------------------------------------
enum { RES_MOMENT = 1, RES_SHEAR = 2, RES_MEMBRANE = 3 };

template <int NN>
FS_HD void resultant_rows(int quant, const double g[NN][2], double c[3][NN][5])
{
    for (int r = 0; r < 3; r++)
        for (int i = 0; i < NN; i++)
            for (int q = 0; q < 5; q++) c[r][i][q] = 0.0;
    for (int i = 0; i < NN; i++) {
        if (quant == RES_MEMBRANE) {
            c[0][i][0] = g[i][0];
            c[1][i][1] = g[i][1];
            c[2][i][0] = g[i][1]; c[2][i][1] = g[i][0];
        } else if (quant == RES_MOMENT) {
            c[0][i][4] = g[i][0];
            c[1][i][3] = -g[i][1];
            c[2][i][3] = -g[i][0]; c[2][i][4] = g[i][1];
        }
    }
}

// cs: the output csys (column-major), or null for the element frame at the
// point -- the shells' default mcsys, whose updater (isoparametric!,
// src/FEMMShellT3FFModule.jl:222-224; _isoparametric!, src/FEMMShellQ4RSModule.jl:
// 201-203) is _e_g! of the point's tangents
template <int NN>
FS_HD void resultant_finish(int quant, const GlobalMap<double, NN> &M, const double e[3][3],
                            const double c[3][NN][5], const double ue[6 * NN], const MatConst &mc, double t,
                            double stab, const double *cs, double out[3])
{
    const int nr = quant == RES_SHEAR ? 2 : 3;
    double s[3] = {0.0, 0.0, 0.0};
    for (int r = 0; r < nr; r++) {
        double row[6 * NN];
        expand_row<double, NN>(M, c[r], row);
        double acc = 0.0;
        for (int k = 0; k < 6 * NN; k++) acc += row[k] * ue[k];
        s[r] = acc;
    }
    double v[3];
    if (quant == RES_SHEAR) {
        const double f = t * stab;
        v[0] = f * (mc.Dt5[0] * s[0] + mc.Dt5[2] * s[1]);
        v[1] = f * (mc.Dt5[1] * s[0] + mc.Dt5[3] * s[1]);
        v[2] = 0.0;
    } else {
        const double f = quant == RES_MOMENT ? (t * t * t) / 12 : t;
        for (int i = 0; i < 3; i++) v[i] = f * (mc.Dps[i] * s[0] + mc.Dps[i + 3] * s[1] + mc.Dps[i + 6] * s[2]);
    }
    // o2 = [m n; -n m]: moments and membrane forces o2' T o2, shear forces o2' f
    double csi[9];
    if (!cs) {
        for (int k = 0; k < 3; k++) {
            csi[k] = e[0][k];
            csi[3 + k] = e[1][k];
            csi[6 + k] = e[2][k];
        }
        cs = csi;
    }
    double m, n;
    layup_angle(e, cs, m, n);
    if (quant == RES_SHEAR) {
        out[0] = m * v[0] - n * v[1];
        out[1] = n * v[0] + m * v[1];
        out[2] = 0.0;
    } else {
        const double t00 = m * v[0] - n * v[2], t01 = m * v[2] - n * v[1];
        const double t10 = n * v[0] + m * v[2], t11 = n * v[2] + m * v[1];
        out[0] = t00 * m - t01 * n;
        out[1] = t10 * n + t11 * m;
        out[2] = t00 * n + t01 * m;
    }
}

// T3FF: one point, the centroid.  ue: the element's 18 global displacements.
FS_HD void t3_resultant(const ElemIn<3> &in, const MatConst &mc, const double ue[18], int quant,
                        const double *cs, double out[3])
{
    double J0[3], J1[3], e[3][3];
    for (int c = 0; c < 3; c++) {
        J0[c] = in.X[1][c] - in.X[0][c];
        J1[c] = in.X[2][c] - in.X[0][c];
    }
    make_frame(J0, J1, e);
    const double a = dot3(J0, e[0]), b = dot3(J0, e[1]);
    const double cc = dot3(J1, e[0]), d = dot3(J1, e[1]);
    const double Jd = a * d - b * cc, Ae = Jd / 2, iJ = 1.0 / Jd;
    double g[3][2];
    g[0][0] = (b - d) * iJ; g[1][0] = d * iJ; g[2][0] = -b * iJ;
    g[0][1] = (cc - a) * iJ; g[1][1] = -cc * iJ; g[2][1] = a * iJ;
    double A[3][3][3];
    for (int i = 0; i < 3; i++) nodal_triad(e, in.nrm[i], in.valid[i], A[i]);
    GlobalMap<double, 3> M;
    build_map<double, 3>(e, A, g, M);
    double c[3][3][5];
    resultant_rows<3>(quant, g, c);
    if (quant == RES_SHEAR) {
        // _Bsmat!: the DSG rows averaged over the three node orderings
        const double x[3] = {0.0, a, cc}, y[3] = {0.0, b, d};
        t3_bs_ordering<double>(x, y, Ae, 0, 1, 2, (double(*)[3][5])c[0], 1.0 / 3);
        t3_bs_ordering<double>(x, y, Ae, 1, 2, 0, (double(*)[3][5])c[0], 1.0 / 3);
        t3_bs_ordering<double>(x, y, Ae, 2, 0, 1, (double(*)[3][5])c[0], 1.0 / 3);
    }
    const double t = in.t;
    const double stab = t * t / (t * t + mc.stab_c * (2 * Ae));
    resultant_finish<3>(quant, M, e, c, ue, mc, t, stab, cs, out);
}

// Q4RS: Gauss point j (0..3, the reference's point order).  Returns nonzero
// on a singular metric (src/FEMMShellQ4RSModule.jl:308-311).
FS_HD int q4_resultant(const ElemIn<4> &in, const Q4Elem &qe, int j, const MatConst &mc,
                       const double ue[24], int quant, const double *cs, double out[3])
{
    double xi, eta, gp[4][2];
    q4_point(j, xi, eta);
    q4_dbasis(xi, eta, gp);
    double J0[3], J1[3];
    for (int c = 0; c < 3; c++) {
        J0[c] = qe.Xr[0][c] * gp[0][0] + qe.Xr[1][c] * gp[1][0] + qe.Xr[2][c] * gp[2][0] + qe.Xr[3][c] * gp[3][0];
        J1[c] = qe.Xr[0][c] * gp[0][1] + qe.Xr[1][c] * gp[1][1] + qe.Xr[2][c] * gp[2][1] + qe.Xr[3][c] * gp[3][1];
    }
    double e[3][3];
    make_frame(J0, J1, e);
    double X[4], Y[4];
    for (int a = 0; a < 4; a++) {
        X[a] = dot3(qe.Xr[a], e[0]);
        Y[a] = dot3(qe.Xr[a], e[1]);
    }
    const double G11 = dot3(J0, J0), G12 = dot3(J0, J1), G22 = dot3(J1, J1);
    const double detG = G11 * G22 - G12 * G12;
    if (detG == 0.0) return 4;
    const double i11 = G22 / detG, i12 = -G12 / detG, i22 = G11 / detG;
    const double pj0[2] = {dot3(e[0], J0), dot3(e[1], J0)}, pj1[2] = {dot3(e[0], J1), dot3(e[1], J1)};
    double g[4][2];
    for (int a = 0; a < 4; a++) {
        const double t1 = i11 * gp[a][0] + i12 * gp[a][1];
        const double t2 = i12 * gp[a][0] + i22 * gp[a][1];
        g[a][0] = pj0[0] * t1 + pj1[0] * t2;
        g[a][1] = pj0[1] * t1 + pj1[1] * t2;
    }
    double A[4][3][3];
    for (int i = 0; i < 4; i++) nodal_triad(e, in.nrm[i], in.valid[i], A[i]);
    GlobalMap<double, 4> M;
    build_map<double, 4>(e, A, g, M);
    double c[3][4][5];
    resultant_rows<4>(quant, g, c);
    if (quant == RES_SHEAR) q4_bs<double>(X, Y, xi, eta, (double(*)[4][5])c[0]);
    resultant_finish<4>(quant, M, e, c, ue, mc, in.t, qe.stab, cs, out);
    return 0;
}

}  // namespace fs

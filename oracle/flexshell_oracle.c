/*
 * CPU oracle for the shell element-assembly hot path.  TEST INFRASTRUCTURE:
 * only tests, the smoke check and the benchmark's CPU-baseline leg use it.
 *
 * Plain-C restatement of FinEtoolsFlexStructures.jl 3.6.4 (reference) and of
 * the FinEtools 8.2.5 helpers it calls (FinEtools itself is not vendored; the
 * helpers are restated from their published behaviour: add_btdb_ut_only!,
 * add_b1tdb2!, complete_lt!, rotmat3!, locjac!, Jacobiansurface, GaussRule,
 * sparse(I,J,V) duplicate summation, SysmatAssemblerSparse/…Symm/…Diag).
 *
 * The formulation is deliberately the reference's dense one (explicit
 * transformation matrices, Q^T E Q congruences) so that it checks the
 * structure-aware CUDA kernels independently.
 */
#include "flexshell_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX(i, j, ld) ((i) + (j) * (ld))

/* ------------------------------------------------------------------ */
/* small dense helpers (column-major)                                  */
/* ------------------------------------------------------------------ */

/* E <- Q^T (E Q), square n x n: TransformerQtEQ, src/TransformerModule.jl:38-42 */
static void qteq(double *E, const double *Q, int n)
{
    double *buf = (double *)malloc(sizeof(double) * n * n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += E[IX(i, k, n)] * Q[IX(k, j, n)];
            buf[IX(i, j, n)] = s;
        }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += Q[IX(k, i, n)] * buf[IX(k, j, n)];
            E[IX(i, j, n)] = s;
        }
    free(buf);
}

/* E <- Q (E Q^T): TransformerQEQt, src/TransformerModule.jl:72-76 */
static void qeqt(double *E, const double *Q, int n)
{
    double buf[9 * 9];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += E[IX(i, k, n)] * Q[IX(j, k, n)];
            buf[IX(i, j, n)] = s;
        }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += Q[IX(i, k, n)] * buf[IX(k, j, n)];
            E[IX(i, j, n)] = s;
        }
}

/* FinEtools add_btdb_ut_only!: upper triangle of K += w B^T D B (B: r x n). */
static void add_btdb_ut(double *K, const double *B, double w, const double *D, int r, int n)
{
    double DB[8 * 24];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < r; i++) {
            double s = 0.0;
            for (int k = 0; k < r; k++) s += D[IX(i, k, r)] * B[IX(k, j, r)];
            DB[IX(i, j, r)] = s * w;
        }
    for (int nx = 0; nx < n; nx++)
        for (int px = 0; px <= nx; px++) {
            double s = 0.0;
            for (int mx = 0; mx < r; mx++) s += B[IX(mx, px, r)] * DB[IX(mx, nx, r)];
            K[IX(px, nx, n)] += s;
        }
}

/* FinEtools add_b1tdb2!: K += w B1^T D B2 (full). */
static void add_b1tdb2(double *K, const double *B1, const double *B2, double w,
                       const double *D, int r, int n)
{
    double DB[8 * 24];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < r; i++) {
            double s = 0.0;
            for (int k = 0; k < r; k++) s += D[IX(i, k, r)] * B2[IX(k, j, r)];
            DB[IX(i, j, r)] = s * w;
        }
    for (int nx = 0; nx < n; nx++)
        for (int px = 0; px < n; px++) {
            double s = 0.0;
            for (int mx = 0; mx < r; mx++) s += B1[IX(mx, px, r)] * DB[IX(mx, nx, r)];
            K[IX(px, nx, n)] += s;
        }
}

/* FinEtools complete_lt!: copy the upper triangle into the lower. */
static void complete_lt(double *K, int n)
{
    for (int j = 0; j < n; j++)
        for (int i = j + 1; i < n; i++) K[IX(i, j, n)] = K[IX(j, i, n)];
}

/* Element frame from the tangent vectors: _e_g!,
 * src/FEMMShellT3FFModule.jl:283-305, src/FEMMShellQ4RSModule.jl:248-264 */
static void e_g(double *E, const double *J)
{
    for (int j = 0; j < 3; j++) E[IX(j, 0, 3)] = J[IX(j, 0, 3)];
    double n = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    for (int j = 0; j < 3; j++) E[IX(j, 0, 3)] /= n;
    E[IX(0, 2, 3)] = -E[IX(2, 0, 3)] * J[IX(1, 1, 3)] + E[IX(1, 0, 3)] * J[IX(2, 1, 3)];
    E[IX(1, 2, 3)] = E[IX(2, 0, 3)] * J[IX(0, 1, 3)] - E[IX(0, 0, 3)] * J[IX(2, 1, 3)];
    E[IX(2, 2, 3)] = -E[IX(1, 0, 3)] * J[IX(0, 1, 3)] + E[IX(0, 0, 3)] * J[IX(1, 1, 3)];
    n = sqrt(E[6] * E[6] + E[7] * E[7] + E[8] * E[8]);
    for (int j = 0; j < 3; j++) E[IX(j, 2, 3)] /= n;
    E[IX(0, 1, 3)] = -E[IX(2, 2, 3)] * E[IX(1, 0, 3)] + E[IX(1, 2, 3)] * E[IX(2, 0, 3)];
    E[IX(1, 1, 3)] = E[IX(2, 2, 3)] * E[IX(0, 0, 3)] - E[IX(0, 2, 3)] * E[IX(2, 0, 3)];
    E[IX(2, 1, 3)] = -E[IX(1, 2, 3)] * E[IX(0, 0, 3)] + E[IX(0, 2, 3)] * E[IX(1, 0, 3)];
}

/* FinEtools rotmat3!: rotation matrix of the rotation vector a
 * (angle |a| about a/|a|): cos(na)(I - a^a^T) + sin(na)/na skew(a) + a^a^T. */
static void rotmat3(double *R, const double *a)
{
    double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (na == 0.0) {
        for (int i = 0; i < 9; i++) R[i] = 0.0;
        R[0] = R[4] = R[8] = 1.0;
        return;
    }
    double S[9] = {0.0, a[2], -a[1], -a[2], 0.0, a[0], a[1], -a[0], 0.0};
    double u[3] = {a[0] / na, a[1] / na, a[2] / na};
    double ca = cos(na), sa = sin(na);
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double aa = u[i] * u[j];
            R[IX(i, j, 3)] = ca * ((i == j ? 1.0 : 0.0) - aa) + sa / na * S[IX(i, j, 3)] + aa;
        }
}

/* _NodalTriadsE, src/FEMMShellT3FFModule.jl:355-388 (same in Q4RS :355-388) */
static void nodal_triads(double *AEs, uint8_t *nv, const double *E, const double *nrm,
                         const uint8_t *valid, int nen)
{
    for (int k = 0; k < nen; k++) {
        double nke[3];
        nv[k] = valid[k];
        if (valid[k]) {
            for (int i = 0; i < 3; i++)
                nke[i] = E[IX(0, i, 3)] * nrm[3 * k + 0] + E[IX(1, i, 3)] * nrm[3 * k + 1] +
                         E[IX(2, i, 3)] * nrm[3 * k + 2];
        } else {
            nke[0] = nke[1] = 0.0;
            nke[2] = 1.0;
        }
        /* r = f3_e x nk_e with f3_e = (0,0,1) */
        double r[3] = {0.0 * nke[2] - 1.0 * nke[1], 1.0 * nke[0] - 0.0 * nke[2],
                       0.0 * nke[1] - 0.0 * nke[0]};
        double *A = AEs + 9 * k;
        if (sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) > 1.0e-12) {
            rotmat3(A, r);
        } else {
            for (int i = 0; i < 9; i++) A[i] = 0.0;
            A[0] = A[4] = A[8] = 1.0;
        }
    }
}

/* _TransfmatGToA, src/FEMMShellT3FFModule.jl:398-419 */
static void transfmat_g_to_a(double *T, const double *AEs, const double *E, int nen)
{
    int n = 6 * nen;
    memset(T, 0, sizeof(double) * n * n);
    for (int i = 0; i < nen; i++) {
        const double *A = AEs + 9 * i;
        double Tb[9];
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) {
                double s = 0.0;
                for (int m = 0; m < 3; m++) s += A[IX(m, r, 3)] * E[IX(c, m, 3)];
                Tb[IX(r, c, 3)] = s;
            }
        int off = 6 * i;
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) {
                T[IX(off + r, off + c, n)] = Tb[IX(r, c, 3)];
                T[IX(off + 3 + r, off + 3 + c, n)] = Tb[IX(r, c, 3)];
            }
    }
}

/* _transfmat_a_to_e!, src/FEMMShellT3FFModule.jl:421-463 */
static void transfmat_a_to_e(double *T, const double *AEs, const double *g, int nen)
{
    int n = 6 * nen;
    memset(T, 0, sizeof(double) * n * n);
    for (int i = 0; i < nen; i++) {
        int ro = 6 * i;
        const double *A = AEs + 9 * i;
        double A33 = A[IX(2, 2, 3)];
        for (int cl = 0; cl < 3; cl++)
            for (int rw = 0; rw < 3; rw++) T[IX(ro + rw, ro + cl, n)] = A[IX(rw, cl, 3)];
        for (int cl = 0; cl < 2; cl++)
            for (int rw = 0; rw < 2; rw++)
                T[IX(ro + 3 + rw, ro + 3 + cl, n)] =
                    A[IX(rw, cl, 3)] - (1.0 / A33) * A[IX(rw, 2, 3)] * A[IX(cl, 2, 3)];
        double m1 = (1.0 / A33) * A[IX(0, 2, 3)];
        double m2 = (1.0 / A33) * A[IX(1, 2, 3)];
        for (int j = 0; j < nen; j++) {
            int co = 6 * j;
            for (int k = 0; k < 3; k++) {
                double a3 = 0.5 * (A[IX(1, k, 3)] * g[IX(j, 0, nen)] - A[IX(0, k, 3)] * g[IX(j, 1, nen)]);
                T[IX(ro + 3, co + k, n)] += m1 * a3;
                T[IX(ro + 4, co + k, n)] += m2 * a3;
            }
        }
    }
}

/* Layup2ElementAngle, src/TransformerModule.jl:92-105 (the square root is
 * clamped at zero where rounding makes 1 - m^2 negative). */
static void layup_angle(const double *E, const double *cs, double *m_out, double *n_out)
{
    double M[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += E[IX(k, i, 3)] * cs[IX(k, j, 3)];
            M[IX(i, j, 3)] = s;
        }
    double a11 = M[IX(0, 0, 3)], a21 = M[IX(1, 0, 3)], a12 = M[IX(0, 1, 3)], a22 = M[IX(1, 1, 3)];
    double n1 = sqrt(a11 * a11 + a21 * a21), n2 = sqrt(a12 * a12 + a22 * a22);
    a11 /= n1; a21 /= n1; a12 /= n2; a22 /= n2;
    double m = (a11 + a22) / 2.0;
    double n = (a12 - a21) / 2.0;
    double sn = (n >= 0.0 ? 1.0 : -1.0);
    double q = 1.0 - m * m;
    n = sn * sqrt(q > 0.0 ? q : 0.0);
    *m_out = m;
    *n_out = n;
}

/* Rotate laminate A,B,D (plane_stress_Tbar_matrix!, src/CompositeLayupModule.jl:364-378)
 * and H (transverse_shear_T_matrix!, :463-471) into the element frame. */
static void rotate_laminate(const double *E, const double *cs, const double *A, const double *B,
                            const double *D, const double *H, double *sA, double *sB,
                            double *sD, double *sH)
{
    double m, n;
    layup_angle(E, cs, &m, &n);
    /* Tinv = [m^2 n^2 2mn; n^2 m^2 -2mn; -mn mn m^2-n^2]; Tbar = Tinv^T */
    double Tb[9];
    Tb[IX(0, 0, 3)] = m * m;       Tb[IX(1, 0, 3)] = n * n;        Tb[IX(2, 0, 3)] = 2 * (m * n);
    Tb[IX(0, 1, 3)] = n * n;       Tb[IX(1, 1, 3)] = m * m;        Tb[IX(2, 1, 3)] = -2 * (m * n);
    Tb[IX(0, 2, 3)] = -(m * n);    Tb[IX(1, 2, 3)] = (m * n);      Tb[IX(2, 2, 3)] = m * m - n * n;
    memcpy(sA, A, 9 * sizeof(double));
    memcpy(sB, B, 9 * sizeof(double));
    memcpy(sD, D, 9 * sizeof(double));
    memcpy(sH, H, 4 * sizeof(double));
    qteq(sA, Tb, 3);
    qteq(sB, Tb, 3);
    qteq(sD, Tb, 3);
    double Tt[4] = {m, n, -n, m}; /* [m -n; n m] column-major */
    qteq(sH, Tt, 2);
}

/* _add_Bsmat_o!, src/FEMMShellT3FFModule.jl:486-526 (0-based nodes s,p,q) */
static void add_bsmat_o(double *Bs, const double *ee, double Ae, int s, int p, int q)
{
    double a = ee[IX(p, 0, 3)] - ee[IX(s, 0, 3)];
    double b = ee[IX(p, 1, 3)] - ee[IX(s, 1, 3)];
    double c = ee[IX(q, 0, 3)] - ee[IX(s, 0, 3)];
    double d = ee[IX(q, 1, 3)] - ee[IX(s, 1, 3)];
    double m = (1.0 / 2.0 / Ae);
    int co = 6 * s;
    Bs[IX(0, co + 2, 2)] += m * (b - d);
    Bs[IX(0, co + 4, 2)] += m * (Ae);
    Bs[IX(1, co + 2, 2)] += m * (c - a);
    Bs[IX(1, co + 3, 2)] += m * (-Ae);
    co = 6 * p;
    Bs[IX(0, co + 2, 2)] += m * (d);
    Bs[IX(0, co + 3, 2)] += m * (-b * d / 2);
    Bs[IX(0, co + 4, 2)] += m * (a * d / 2);
    Bs[IX(1, co + 2, 2)] += m * (-c);
    Bs[IX(1, co + 3, 2)] += m * (b * c / 2);
    Bs[IX(1, co + 4, 2)] += m * (-a * c / 2);
    co = 6 * q;
    Bs[IX(0, co + 2, 2)] += m * (-b);
    Bs[IX(0, co + 3, 2)] += m * (b * d / 2);
    Bs[IX(0, co + 4, 2)] += m * (-b * c / 2);
    Bs[IX(1, co + 2, 2)] += m * (a);
    Bs[IX(1, co + 3, 2)] += m * (-a * d / 2);
    Bs[IX(1, co + 4, 2)] += m * (a * c / 2);
}

static double stab_fun(double t, double h, double c) { return t * t / (t * t + c * h * h); }

static int is_comp(int et) { return et == ORC_T3FFCOMP || et == ORC_Q4RSCOMP; }
static int nen_of(int et) { return (et == ORC_T3FF || et == ORC_T3FFCOMP) ? 3 : 4; }

/* Element material in the element frame: homogeneous -> A = t Dps etc.,
 * composite -> group laminate rotated by the layup angle. */
static void elem_thickness(const orc_params *p, int64_t e, double *t)
{
    if (is_comp(p->etype)) *t = p->gthick[p->group[e]];
    else *t = p->thickness[e];
}

/* ------------------------------------------------------------------ */
/* T3FF / T3FFComp element stiffness                                   */
/* src/FEMMShellT3FFModule.jl:670-731, src/FEMMShellT3FFCompModule.jl:606-682 */
/* ------------------------------------------------------------------ */
static int t3_stiffness(const orc_params *p, int64_t e, const double *X, const double *nrm,
                        const uint8_t *valid, double *K)
{
    const int n = 18;
    double J0[6], E[9], ee[6], g[6];
    for (int j = 0; j < 3; j++) {
        J0[IX(j, 0, 3)] = X[3 * 1 + j] - X[3 * 0 + j];
        J0[IX(j, 1, 3)] = X[3 * 2 + j] - X[3 * 0 + j];
    }
    e_g(E, J0);
    ee[IX(0, 0, 3)] = ee[IX(0, 1, 3)] = 0.0;
    ee[IX(1, 0, 3)] = J0[0] * E[0] + J0[1] * E[1] + J0[2] * E[2];
    ee[IX(1, 1, 3)] = J0[0] * E[3] + J0[1] * E[4] + J0[2] * E[5];
    ee[IX(2, 0, 3)] = J0[3] * E[0] + J0[4] * E[1] + J0[5] * E[2];
    ee[IX(2, 1, 3)] = J0[3] * E[3] + J0[4] * E[4] + J0[5] * E[5];
    double a = ee[IX(1, 0, 3)] - ee[IX(0, 0, 3)], b = ee[IX(1, 1, 3)] - ee[IX(0, 1, 3)];
    double c = ee[IX(2, 0, 3)] - ee[IX(0, 0, 3)], d = ee[IX(2, 1, 3)] - ee[IX(0, 1, 3)];
    double J = a * d - b * c;
    g[IX(0, 0, 3)] = (b - d) / J; g[IX(1, 0, 3)] = d / J; g[IX(2, 0, 3)] = -b / J;
    g[IX(0, 1, 3)] = (c - a) / J; g[IX(1, 1, 3)] = -c / J; g[IX(2, 1, 3)] = a / J;
    double Ae = J / 2;
    double t;
    elem_thickness(p, e, &t);

    memset(K, 0, sizeof(double) * n * n);
    double Bm[3 * 18] = {0}, Bb[3 * 18] = {0}, Bs[2 * 18];
    for (int i = 0; i < 3; i++) {
        Bm[IX(0, 6 * i + 0, 3)] = g[IX(i, 0, 3)];
        Bm[IX(1, 6 * i + 1, 3)] = g[IX(i, 1, 3)];
        Bm[IX(2, 6 * i + 0, 3)] = g[IX(i, 1, 3)];
        Bm[IX(2, 6 * i + 1, 3)] = g[IX(i, 0, 3)];
        Bb[IX(0, 6 * i + 4, 3)] = g[IX(i, 0, 3)];
        Bb[IX(1, 6 * i + 3, 3)] = -g[IX(i, 1, 3)];
        Bb[IX(2, 6 * i + 3, 3)] = -g[IX(i, 0, 3)];
        Bb[IX(2, 6 * i + 4, 3)] = g[IX(i, 1, 3)];
    }
    double h = sqrt(2 * Ae);
    double Hs[4], wshear;
    if (!is_comp(p->etype)) {
        add_btdb_ut(K, Bm, t * Ae, p->Dps, 3, n);
        add_btdb_ut(K, Bb, (t * t * t) / 12 * Ae, p->Dps, 3, n);
        for (int i = 0; i < 4; i++) Hs[i] = p->Dt[i] * (5.0 / 6.0);
        wshear = t * stab_fun(t, h, p->stab_c) * Ae;
    } else {
        int gi = p->group[e];
        double sA[9], sB[9], sD[9], sH[4];
        rotate_laminate(E, p->gcsmat + 9 * gi, p->gA + 9 * gi, p->gB + 9 * gi, p->gD + 9 * gi,
                        p->gH + 4 * gi, sA, sB, sD, sH);
        add_btdb_ut(K, Bm, Ae, sA, 3, n);
        add_btdb_ut(K, Bb, Ae, sD, 3, n);
        add_b1tdb2(K, Bm, Bb, Ae, sB, 3, n);
        add_b1tdb2(K, Bb, Bm, Ae, sB, 3, n);
        memcpy(Hs, sH, sizeof(sH));
        wshear = stab_fun(t, h, p->stab_c) * Ae;
    }
    if (p->tsf == 1) {
        static const int ord[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
        for (int o = 0; o < 3; o++) {
            memset(Bs, 0, sizeof(Bs));
            add_bsmat_o(Bs, ee, Ae, ord[o][0], ord[o][1], ord[o][2]);
            add_btdb_ut(K, Bs, wshear / 3, Hs, 2, n);
        }
    } else {
        memset(Bs, 0, sizeof(Bs));
        add_bsmat_o(Bs, ee, Ae, 0, 1, 2);
        add_bsmat_o(Bs, ee, Ae, 1, 2, 0);
        add_bsmat_o(Bs, ee, Ae, 2, 0, 1);
        for (int i = 0; i < 36; i++) Bs[i] *= (1.0 / 3);
        add_btdb_ut(K, Bs, wshear, Hs, 2, n);
    }
    complete_lt(K, n);

    double AEs[27], T[18 * 18];
    uint8_t nv[3];
    nodal_triads(AEs, nv, E, nrm, valid, 3);
    transfmat_a_to_e(T, AEs, g, 3);
    qteq(K, T, n);
    double kavg = (K[IX(3, 3, n)] + K[IX(9, 9, n)] + K[IX(15, 15, n)] + K[IX(4, 4, n)] +
                   K[IX(10, 10, n)] + K[IX(16, 16, n)]) / 6.0 * p->drill_scale;
    for (int k = 0; k < 3; k++)
        if (nv[k]) K[IX(6 * k + 5, 6 * k + 5, n)] += kavg;
    transfmat_g_to_a(T, AEs, E, 3);
    qteq(K, T, n);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Q4RS / Q4RSComp element stiffness                                   */
/* src/FEMMShellQ4RSModule.jl:913-944, src/FEMMShellQ4RSCompModule.jl:908-951 */
/* ------------------------------------------------------------------ */

/* FinEtools GaussRule(2,2) (points in i-outer, j-inner order, weights 1)
 * and the bilinear Q4 basis (node k at (xi,eta) = corners counterclockwise). */
static const double GP = 0.577350269189626;
static void q4_point(int j, double *xi, double *eta)
{
    static const double s[4][2] = {{-1, -1}, {-1, 1}, {1, -1}, {1, 1}};
    *xi = s[j][0] * GP;
    *eta = s[j][1] * GP;
}
static void q4_basis(double xi, double eta, double *N, double *gp /* 4x2 col-major */)
{
    N[0] = 0.25 * (1 - xi) * (1 - eta);
    N[1] = 0.25 * (1 + xi) * (1 - eta);
    N[2] = 0.25 * (1 + xi) * (1 + eta);
    N[3] = 0.25 * (1 - xi) * (1 + eta);
    gp[IX(0, 0, 4)] = -0.25 * (1 - eta); gp[IX(0, 1, 4)] = -0.25 * (1 - xi);
    gp[IX(1, 0, 4)] = 0.25 * (1 - eta);  gp[IX(1, 1, 4)] = -0.25 * (1 + xi);
    gp[IX(2, 0, 4)] = 0.25 * (1 + eta);  gp[IX(2, 1, 4)] = 0.25 * (1 + xi);
    gp[IX(3, 0, 4)] = -0.25 * (1 + eta); gp[IX(3, 1, 4)] = 0.25 * (1 - xi);
}

/* locjac!: J = X^T gradNparams (3x2) */
static void q4_jac(const double *X, const double *gp, double *J)
{
    for (int k = 0; k < 2; k++)
        for (int c = 0; c < 3; c++) {
            double s = 0.0;
            for (int a = 0; a < 4; a++) s += X[3 * a + c] * gp[IX(a, k, 4)];
            J[IX(c, k, 3)] = s;
        }
}

static double cross_norm(const double *J)
{
    double x = J[1] * J[5] - J[2] * J[4];
    double y = J[2] * J[3] - J[0] * J[5];
    double z = J[0] * J[4] - J[1] * J[3];
    return sqrt(x * x + y * y + z * z);
}

/* _Bsmat (MITC, Bathe-Dvorkin), src/FEMMShellQ4RSModule.jl:702-751; result in
 * element-frame dofs (2 x 24). */
static void q4_bs_elem(double *Bs, const double *ee /* 4x2 */, double r, double s)
{
    memset(Bs, 0, sizeof(double) * 48);
    double X1 = ee[IX(0, 0, 4)], Y1 = ee[IX(0, 1, 4)];
    double X2 = ee[IX(1, 0, 4)], Y2 = ee[IX(1, 1, 4)];
    double X3 = ee[IX(2, 0, 4)], Y3 = ee[IX(2, 1, 4)];
    double X4 = ee[IX(3, 0, 4)], Y4 = ee[IX(3, 1, 4)];
    double J11 = (X1 * (s - 1) / 4 - X2 * (s - 1) / 4 + X3 * (s + 1) / 4 - X4 * (s + 1) / 4);
    double J21 = (Y1 * (s - 1) / 4 - Y2 * (s - 1) / 4 + Y3 * (s + 1) / 4 - Y4 * (s + 1) / 4);
    double J12 = (X1 * (r - 1) / 4 - X2 * (r + 1) / 4 + X3 * (r + 1) / 4 - X4 * (r - 1) / 4);
    double J22 = (Y1 * (r - 1) / 4 - Y2 * (r + 1) / 4 + Y3 * (r + 1) / 4 - Y4 * (r - 1) / 4);
    double A = sqrt(J11 * J11 + J21 * J21), B = sqrt(J12 * J12 + J22 * J22);
    double ca = J11 / A, sa = J21 / A, cb = J12 / B, sb = J22 / B;
    double detJ = J11 * J22 - J12 * J21;
    double Ax = X1 - X2 - X3 + X4, Ay = Y1 - Y2 - Y3 + Y4;
    double Bx = X1 - X2 + X3 - X4, By = Y1 - Y2 + Y3 - Y4;
    double Cx = X1 + X2 - X3 - X4, Cy = Y1 + Y2 - Y3 - Y4;
    double LA = sqrt((Ax + Bx * s) * (Ax + Bx * s) + (Ay + By * s) * (Ay + By * s));
    double LB = sqrt((Bx * r + Cx) * (Bx * r + Cx) + (By * r + Cy) * (By * r + Cy));
    /* row 0 (gxz) uses (p,q) = (sa, sb); row 1 (gyz) uses (-ca, -cb) */
    for (int row = 0; row < 2; row++) {
        double pp = row == 0 ? sa : -ca;
        double qq = row == 0 ? sb : -cb;
        double fa = pp * LA, fb = qq * LB;
        double *R = Bs + row; /* stride 2 */
#define BS(col) R[2 * (col)]
        BS(2) += (fa * (r + 1) - fb * (s + 1)) / (16 * detJ);
        BS(3) += (-fa * (Y1 - Y4) * (r + 1) + fb * (Y1 - Y2) * (s + 1)) / (32 * detJ);
        BS(4) += (fa * (X1 - X4) * (r + 1) - fb * (X1 - X2) * (s + 1)) / (32 * detJ);
        BS(8) += (-fa * (r - 1) + fb * (s + 1)) / (16 * detJ);
        BS(9) += (fa * (Y2 - Y3) * (r - 1) + fb * (Y1 - Y2) * (s + 1)) / (32 * detJ);
        BS(10) += (-fa * (X2 - X3) * (r - 1) - fb * (X1 - X2) * (s + 1)) / (32 * detJ);
        BS(14) += (fa * (r - 1) - fb * (s - 1)) / (16 * detJ);
        BS(15) += (fa * (Y2 - Y3) * (r - 1) + fb * (Y3 - Y4) * (s - 1)) / (32 * detJ);
        BS(16) += (-fa * (X2 - X3) * (r - 1) - fb * (X3 - X4) * (s - 1)) / (32 * detJ);
        BS(20) += (-fa * (r + 1) + fb * (s - 1)) / (16 * detJ);
        BS(21) += (-fa * (Y1 - Y4) * (r + 1) + fb * (Y3 - Y4) * (s - 1)) / (32 * detJ);
        BS(22) += (fa * (X1 - X4) * (r + 1) - fb * (X3 - X4) * (s - 1)) / (32 * detJ);
#undef BS
    }
}

static void matmul_rn(const double *A, int r, int k, const double *B, int n, double *C)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < r; i++) {
            double s = 0.0;
            for (int m = 0; m < k; m++) s += A[IX(i, m, r)] * B[IX(m, j, k)];
            C[IX(i, j, r)] = s;
        }
}

static double q4_diameter(const double *X)
{
    double mx = 0.0;
    for (int i = 1; i < 4; i++) {
        double dx = X[3 * i] - X[0], dy = X[3 * i + 1] - X[1], dz = X[3 * i + 2] - X[2];
        double d = dx * dx + dy * dy + dz * dz;
        if (d > mx) mx = d;
    }
    return sqrt(mx);
}

static int q4_stiffness(const orc_params *p, int64_t e, const double *X, const double *nrm,
                        const uint8_t *valid, double *K)
{
    const int n = 24;
    double t;
    elem_thickness(p, e, &t);
    double h = q4_diameter(X);
    memset(K, 0, sizeof(double) * n * n);
    double Dt5[4];
    for (int i = 0; i < 4; i++) Dt5[i] = p->Dt[i] * (5.0 / 6.0);
    double *T = (double *)malloc(sizeof(double) * 3 * n * n);
    double *Tae = T + n * n, *Tga = T + 2 * n * n;
    for (int j = 0; j < 4; j++) {
        double xi, eta, N[4], gp[8], J[6], E[9], ee[8], g[8];
        q4_point(j, &xi, &eta);
        q4_basis(xi, eta, N, gp);
        q4_jac(X, gp, J);
        double Jac = cross_norm(J);
        e_g(E, J);
        /* _EcoordsE: centroid-relative coordinates on the element basis */
        double cen[3] = {0, 0, 0};
        for (int a = 0; a < 4; a++)
            for (int k = 0; k < 3; k++) cen[k] += X[3 * a + k];
        for (int k = 0; k < 3; k++) cen[k] /= 4;
        for (int a = 0; a < 4; a++)
            for (int k = 0; k < 2; k++) {
                double d = 0.0;
                for (int m = 0; m < 3; m++) d += (X[3 * a + m] - cen[m]) * E[IX(m, k, 3)];
                ee[IX(a, k, 4)] = d;
            }
        /* _LocalDerivatives: metric inverse, src/FEMMShellQ4RSModule.jl:305-323 */
        double G11 = J[0] * J[0] + J[1] * J[1] + J[2] * J[2];
        double G12 = J[0] * J[3] + J[1] * J[4] + J[2] * J[5];
        double G22 = J[3] * J[3] + J[4] * J[4] + J[5] * J[5];
        double detG = G11 * G22 - G12 * G12;
        if (detG == 0.0) {
            free(T);
            return 4; /* singular metric */
        }
        double i11 = G22 / detG, i12 = -G12 / detG, i22 = G11 / detG;
        for (int a = 0; a < 4; a++) {
            double t1 = i11 * gp[IX(a, 0, 4)] + i12 * gp[IX(a, 1, 4)];
            double t2 = i12 * gp[IX(a, 0, 4)] + i22 * gp[IX(a, 1, 4)];
            double v[3];
            for (int c = 0; c < 3; c++) v[c] = J[IX(c, 0, 3)] * t1 + J[IX(c, 1, 3)] * t2;
            g[IX(a, 0, 4)] = E[0] * v[0] + E[1] * v[1] + E[2] * v[2];
            g[IX(a, 1, 4)] = E[3] * v[0] + E[4] * v[1] + E[5] * v[2];
        }
        double AEs[36];
        uint8_t nv[4];
        nodal_triads(AEs, nv, E, nrm, valid, 4);
        transfmat_g_to_a(Tga, AEs, E, 4);
        transfmat_a_to_e(Tae, AEs, g, 4);
        matmul_rn(Tae, n, n, Tga, n, T);
        double tBm[3 * 24] = {0}, tBb[3 * 24] = {0}, tBs[2 * 24];
        for (int i = 0; i < 4; i++) {
            int off = 6 * i;
            tBm[IX(0, off + 0, 3)] = g[IX(i, 0, 4)];
            tBm[IX(1, off + 1, 3)] = g[IX(i, 1, 4)];
            tBm[IX(2, off + 0, 3)] = g[IX(i, 1, 4)];
            tBm[IX(2, off + 1, 3)] = g[IX(i, 0, 4)];
            tBb[IX(0, off + 4, 3)] = g[IX(i, 0, 4)];
            tBb[IX(1, off + 3, 3)] = -g[IX(i, 1, 4)];
            tBb[IX(2, off + 3, 3)] = -g[IX(i, 0, 4)];
            tBb[IX(2, off + 4, 3)] = g[IX(i, 1, 4)];
        }
        double Bm[3 * 24], Bb[3 * 24], Bs[2 * 24];
        matmul_rn(tBm, 3, n, T, n, Bm);
        matmul_rn(tBb, 3, n, T, n, Bb);
        q4_bs_elem(tBs, ee, xi, eta);
        matmul_rn(tBs, 2, n, T, n, Bs);
        double w = 1.0;
        if (!is_comp(p->etype)) {
            add_btdb_ut(K, Bm, t * Jac * w, p->Dps, 3, n);
            add_btdb_ut(K, Bb, (t * t * t / 12.0) * Jac * w, p->Dps, 3, n);
            add_btdb_ut(K, Bs, t * stab_fun(t, h, p->stab_c) * Jac * w, Dt5, 2, n);
        } else {
            int gi = p->group[e];
            double sA[9], sB[9], sD[9], sH[4];
            rotate_laminate(E, p->gcsmat + 9 * gi, p->gA + 9 * gi, p->gB + 9 * gi, p->gD + 9 * gi,
                            p->gH + 4 * gi, sA, sB, sD, sH);
            add_btdb_ut(K, Bm, Jac * w, sA, 3, n);
            add_btdb_ut(K, Bb, Jac * w, sD, 3, n);
            add_b1tdb2(K, Bm, Bb, Jac * w, sB, 3, n);
            add_b1tdb2(K, Bb, Bm, Jac * w, sB, 3, n);
            add_btdb_ut(K, Bs, stab_fun(t, h, p->stab_c) * Jac * w, sH, 2, n);
        }
    }
    free(T);
    complete_lt(K, n);
    /* _add_drilling_stiffness!, src/FEMMShellQ4RSModule.jl:807-859 */
    if (p->drill_scale != 0.0) {
        double sum = 0.0;
        int cnt = 0;
        for (int k = 0; k < 4; k++) {
            if (!valid[k]) continue;
            const double *nv = nrm + 3 * k;
            double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
            if (nn == 0.0) continue;
            double u[3] = {nv[0] / nn, nv[1] / nn, nv[2] / nn};
            int r0 = 6 * k + 3;
            double P[9], PK[9], tr = 0.0;
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) P[IX(i, j, 3)] = (i == j ? 1.0 : 0.0) - u[i] * u[j];
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                    double s = 0.0;
                    for (int m = 0; m < 3; m++) s += P[IX(i, m, 3)] * K[IX(r0 + m, r0 + j, n)];
                    PK[IX(i, j, 3)] = s;
                }
            for (int i = 0; i < 3; i++) {
                double s = 0.0;
                for (int m = 0; m < 3; m++) s += PK[IX(i, m, 3)] * P[IX(m, i, 3)];
                tr += s;
            }
            double v = tr / 2.0;
            sum += (v > 0.0 ? v : 0.0);
            cnt++;
        }
        double kavg = (cnt ? sum / cnt : 0.0) * p->drill_scale;
        if (kavg != 0.0) {
            for (int k = 0; k < 4; k++) {
                if (!valid[k]) continue;
                const double *nv = nrm + 3 * k;
                if (sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]) == 0.0) continue;
                int r0 = 6 * k + 3;
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++) K[IX(r0 + i, r0 + j, n)] += kavg * (nv[i] * nv[j]);
            }
        }
    }
    return 0;
}

int orc_element_stiffness(const orc_params *p, int64_t e, const double *X, const double *nrm,
                          const uint8_t *nvalid, double *Ke)
{
    if (nen_of(p->etype) == 3) return t3_stiffness(p, e, X, nrm, nvalid, Ke);
    return q4_stiffness(p, e, X, nrm, nvalid, Ke);
}

/* Lumped mass: src/FEMMShellT3FFModule.jl:770-787, src/FEMMShellQ4RSModule.jl:981-997,
 * src/FEMMShellT3FFCompModule.jl:731-748, src/FEMMShellQ4RSCompModule.jl:1000-1015 */
int orc_element_mass(const orc_params *p, int64_t e, const double *X, double *tm, double *rm)
{
    double t;
    elem_thickness(p, e, &t);
    int comp = is_comp(p->etype);
    double md = comp ? p->gmass[p->group[e]] : 0.0, mi = comp ? p->gmoi[p->group[e]] : 0.0;
    if (nen_of(p->etype) == 3) {
        double J0[6], E[9];
        for (int j = 0; j < 3; j++) {
            J0[IX(j, 0, 3)] = X[3 * 1 + j] - X[j];
            J0[IX(j, 1, 3)] = X[3 * 2 + j] - X[j];
        }
        e_g(E, J0);
        double a = J0[0] * E[0] + J0[1] * E[1] + J0[2] * E[2];
        double b = J0[0] * E[3] + J0[1] * E[4] + J0[2] * E[5];
        double c = J0[3] * E[0] + J0[4] * E[1] + J0[5] * E[2];
        double d = J0[3] * E[3] + J0[4] * E[4] + J0[5] * E[5];
        double Ae = (a * d - b * c) / 2;
        if (comp) {
            *tm = md * (Ae / 3);
            *rm = mi * (Ae / 3);
        } else {
            *tm = p->rho * (t * Ae) / 3;
            *rm = p->rho * (t * t * t / 12 * Ae) / 3;
        }
    } else {
        double ts = 0.0, rs = 0.0;
        for (int j = 0; j < 4; j++) {
            double xi, eta, N[4], gp[8], J[6];
            q4_point(j, &xi, &eta);
            q4_basis(xi, eta, N, gp);
            q4_jac(X, gp, J);
            double Jac = cross_norm(J);
            if (comp) {
                ts += md * Jac * 1.0;
                rs += mi * Jac * 1.0;
            } else {
                ts += p->rho * t * Jac * 1.0;
                rs += p->rho * t * t * t / 12 * Jac * 1.0;
            }
        }
        *tm = ts / 4;
        *rm = rs / 4;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Nodal normals: associategeometry!, src/FEMMShellT3FFModule.jl:570-616,   */
/* src/FEMMShellQ4RSModule.jl:472-525 and the Comp variants (the layup       */
/* csys third axis replaces the isoparametric normal).                      */
/* ------------------------------------------------------------------ */
static void gather_X(const double *xyz, int64_t nnodes, const int64_t *cn, int nen, double *X)
{
    for (int a = 0; a < nen; a++)
        for (int c = 0; c < 3; c++) X[3 * a + c] = xyz[(cn[a] - 1) + c * nnodes];
}

/* The third axis of the built-in material csys kinds at the point XYZ: the
 * csys updaters of the reference examples, generalised (cartesian! of
 * bent_strip_examples.jl:15-20: a fixed matrix; cylindrical! of
 * clamp_cyl_expl_examples.jl:61-67: radial from an axis, there the y axis;
 * spherical! of hemisphere_examples.jl:31-39: radial from a centre, there the
 * origin).  params: CARTESIAN the 3x3 column-major matrix; CYLINDRICAL a
 * point on the axis and the unit axis direction; SPHERICAL the centre. */
static void csys_normal(int kind, const double *prm, const double *XYZ, double *nn)
{
    double r[3];
    if (kind == ORC_CSYS_CARTESIAN) {
        nn[0] = prm[6]; nn[1] = prm[7]; nn[2] = prm[8];
        return;
    }
    for (int c = 0; c < 3; c++) r[c] = XYZ[c] - prm[c];
    if (kind == ORC_CSYS_CYLINDRICAL) {
        double d = r[0] * prm[3] + r[1] * prm[4] + r[2] * prm[5];
        for (int c = 0; c < 3; c++) r[c] -= d * prm[3 + c];
    }
    double l = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int c = 0; c < 3; c++) nn[c] = r[c] / l;
}

static void point_normal(const orc_params *p, int64_t e, const double *X, int j, double *nn,
                         double *Jac, int kind, const double *prm)
{
    int nen = nen_of(p->etype);
    double J[6], E[9];
    if (nen == 3) {
        for (int c = 0; c < 3; c++) {
            J[IX(c, 0, 3)] = X[3 + c] - X[c];
            J[IX(c, 1, 3)] = X[6 + c] - X[c];
        }
        *Jac = 1.0;
    } else {
        static const double nodes[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        double N[4], gp[8];
        q4_basis(nodes[j][0], nodes[j][1], N, gp);
        q4_jac(X, gp, J);
        *Jac = cross_norm(J);
    }
    if (is_comp(p->etype)) {
        const double *cs = p->gcsmat + 9 * p->group[e];
        nn[0] = cs[6]; nn[1] = cs[7]; nn[2] = cs[8];
    } else if (kind != ORC_CSYS_ISOPARAMETRIC) {
        csys_normal(kind, prm, X + 3 * j, nn);  /* at the node: loc of the nodal rule */
    } else {
        e_g(E, J);
        nn[0] = E[6]; nn[1] = E[7]; nn[2] = E[8];
    }
}

int orc_normals(int etype, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                const int64_t *order, double threshold_deg, const orc_params *p, double *normals,
                uint8_t *valid)
{
    return orc_normals_csys(etype, nnodes, xyz, nelem, conn, order, threshold_deg, p, ORC_CSYS_ISOPARAMETRIC,
                            NULL, normals, valid);
}

/* The same with the material csys of one of the built-in kinds: the node sums
 * use the csys normal at the node (weighted by the Jacobian for Q4); the
 * validity test compares with the element frame normal for T3
 * (src/FEMMShellT3FFModule.jl:598-611) and with the csys normal for Q4
 * (src/FEMMShellQ4RSModule.jl:505-519). */
int orc_normals_csys(int etype, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                     const int64_t *order, double threshold_deg, const orc_params *p, int kind,
                     const double *prm, double *normals, uint8_t *valid)
{
    (void)etype;
    int nen = nen_of(p->etype);
    for (int64_t i = 0; i < 3 * nnodes; i++) normals[i] = 0.0;
    for (int64_t i = 0; i < nnodes; i++) valid[i] = 1;
    for (int64_t r = 0; r < nelem; r++) {
        int64_t e = order ? order[r] : r;
        const int64_t *cn = conn + nen * e;
        double X[12];
        gather_X(xyz, nnodes, cn, nen, X);
        for (int j = 0; j < nen; j++) {
            double nn[3], Jac;
            point_normal(p, e, X, j, nn, &Jac, kind, prm);
            int64_t node = cn[j] - 1;
            for (int c = 0; c < 3; c++) normals[node + c * nnodes] += (nen == 3 ? nn[c] : Jac * nn[c]);
        }
    }
    for (int64_t i = 0; i < nnodes; i++) {
        double x = normals[i], y = normals[i + nnodes], z = normals[i + 2 * nnodes];
        double nn = sqrt(x * x + y * y + z * z);
        if (nn > 0.0) {
            normals[i] /= nn;
            normals[i + nnodes] /= nn;
            normals[i + 2 * nnodes] /= nn;
        }
    }
    double sn = sin(threshold_deg / 180 * M_PI);
    double ntol = 1 - sqrt(1 - sn * sn);
    for (int64_t r = 0; r < nelem; r++) {
        int64_t e = order ? order[r] : r;
        const int64_t *cn = conn + nen * e;
        double X[12];
        gather_X(xyz, nnodes, cn, nen, X);
        for (int j = 0; j < nen; j++) {
            double nn[3], Jac;
            point_normal(p, e, X, j, nn, &Jac, nen == 3 ? ORC_CSYS_ISOPARAMETRIC : kind, prm);
            int64_t node = cn[j] - 1;
            double nd = normals[node] * nn[0] + normals[node + nnodes] * nn[1] +
                        normals[node + 2 * nnodes] * nn[2];
            if (nd < 1 - ntol) valid[node] = 0;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Assembly semantics                                                  */
/* ------------------------------------------------------------------ */
struct orc_result {
    int64_t n, nnz;
    int64_t *colptr, *rowval;
    double *nzval;
};

/* Julia sparse(I,J,V,n,n) with duplicates combined by + in the order of
 * appearance; explicit zeros retained.  Output CSC (0-based internally). */
static void coo_to_csc(int64_t n, int64_t m, const int64_t *I, const int64_t *J, const double *V,
                       int64_t **cp_out, int64_t **rv_out, double **nz_out, int64_t *nnz_out)
{
    int64_t *cnt = (int64_t *)calloc(n + 1, sizeof(int64_t));
    int64_t *p1 = (int64_t *)malloc(sizeof(int64_t) * (m > 0 ? m : 1));
    int64_t *p2 = (int64_t *)malloc(sizeof(int64_t) * (m > 0 ? m : 1));
    /* stable counting sort by row */
    for (int64_t k = 0; k < m; k++) cnt[I[k] + 1]++;
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    for (int64_t k = 0; k < m; k++) p1[cnt[I[k]]++] = k;
    /* stable counting sort by column */
    memset(cnt, 0, sizeof(int64_t) * (n + 1));
    for (int64_t k = 0; k < m; k++) cnt[J[k] + 1]++;
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    memcpy(start, cnt, sizeof(int64_t) * (n + 1));
    for (int64_t q = 0; q < m; q++) {
        int64_t k = p1[q];
        p2[cnt[J[k]]++] = k;
    }
    /* combine duplicates: within a column entries are row-sorted and, for
     * equal rows, in the order of appearance */
    int64_t *cp = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    int64_t *rv = (int64_t *)malloc(sizeof(int64_t) * (m > 0 ? m : 1));
    double *nz = (double *)malloc(sizeof(double) * (m > 0 ? m : 1));
    int64_t w = 0;
    for (int64_t c = 0; c < n; c++) {
        cp[c] = w;
        int64_t last = -1;
        for (int64_t q = start[c]; q < start[c + 1]; q++) {
            int64_t k = p2[q];
            if (I[k] == last) {
                nz[w - 1] = nz[w - 1] + V[k];
            } else {
                rv[w] = I[k];
                nz[w] = V[k];
                last = I[k];
                w++;
            }
        }
    }
    cp[n] = w;
    free(cnt); free(p1); free(p2); free(start);
    *cp_out = cp; *rv_out = rv; *nz_out = nz; *nnz_out = w;
}

/* S + transpose(S) with zero results dropped, then the diagonal halved:
 * FinEtools SysmatAssemblerSparseSymm makematrix!. */
static void symm_complete(int64_t n, int64_t *cp, int64_t *rv, double *nz, int64_t **cpo,
                          int64_t **rvo, double **nzo, int64_t *nnzo)
{
    int64_t nnz = cp[n];
    /* transpose */
    int64_t *tcp = (int64_t *)calloc(n + 1, sizeof(int64_t));
    int64_t *trv = (int64_t *)malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
    double *tnz = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    for (int64_t k = 0; k < nnz; k++) tcp[rv[k] + 1]++;
    for (int64_t i = 0; i < n; i++) tcp[i + 1] += tcp[i];
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    memcpy(pos, tcp, sizeof(int64_t) * (n + 1));
    for (int64_t c = 0; c < n; c++)
        for (int64_t k = cp[c]; k < cp[c + 1]; k++) {
            int64_t q = pos[rv[k]]++;
            trv[q] = c;
            tnz[q] = nz[k];
        }
    int64_t *ocp = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
    int64_t *orv = (int64_t *)malloc(sizeof(int64_t) * (2 * nnz > 0 ? 2 * nnz : 1));
    double *onz = (double *)malloc(sizeof(double) * (2 * nnz > 0 ? 2 * nnz : 1));
    int64_t w = 0;
    for (int64_t c = 0; c < n; c++) {
        ocp[c] = w;
        int64_t a = cp[c], ae = cp[c + 1], b = tcp[c], be = tcp[c + 1];
        while (a < ae || b < be) {
            int64_t r;
            double v;
            if (b >= be || (a < ae && rv[a] < trv[b])) {
                r = rv[a]; v = nz[a]; a++;
            } else if (a >= ae || trv[b] < rv[a]) {
                r = trv[b]; v = tnz[b]; b++;
            } else {
                r = rv[a]; v = nz[a] + tnz[b]; a++; b++;
            }
            if (v != 0.0) {
                if (r == c) v /= 2.0;
                orv[w] = r;
                onz[w] = v;
                w++;
            }
        }
    }
    ocp[n] = w;
    free(tcp); free(trv); free(tnz); free(pos);
    *cpo = ocp; *rvo = orv; *nzo = onz; *nnzo = w;
}

int orc_all_element_stiffness(int64_t nnodes, const double *xyz, int64_t nelem,
                              const int64_t *conn, const double *normals, const uint8_t *valid,
                              const orc_params *p, int nthreads, double *Ke_all)
{
    int nen = nen_of(p->etype), nd = 6 * nen;
    int status = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) reduction(| : status)
#endif
    for (int64_t e = 0; e < nelem; e++) {
        const int64_t *cn = conn + nen * e;
        double X[12], nr[12];
        uint8_t vl[4];
        gather_X(xyz, nnodes, cn, nen, X);
        for (int a = 0; a < nen; a++) {
            int64_t node = cn[a] - 1;
            for (int c = 0; c < 3; c++) nr[3 * a + c] = normals[node + c * nnodes];
            vl[a] = valid[node];
        }
        status |= orc_element_stiffness(p, e, X, nr, vl, Ke_all + (int64_t)nd * nd * e);
    }
    (void)nthreads;
    return status;
}

/* Check helper for meshes too large for a COO buffer: the oracle's element
 * stiffness matrices (orc_element_stiffness, the reference loop) of every
 * element, summed into the values of a given 1-based CSC pattern (colptr,
 * rowval) of size n; dofs above n are left out, as the assemblers do.
 * touched[k] is set for every stored entry that receives a contribution and
 * *missing counts contributions whose (row, column) the pattern lacks, so a
 * pattern equal to the oracle's union pattern gives missing 0 and every entry
 * touched.  Sums run in no fixed order (OpenMP over elements, atomic adds):
 * for comparisons at a relative tolerance, not bitwise. */
int orc_csc_accumulate_stiffness(int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                                 const double *normals, const uint8_t *valid, const orc_params *p,
                                 const int64_t *dofnums, int64_t n, const int64_t *colptr,
                                 const int64_t *rowval, double *vals, uint8_t *touched, int64_t *missing,
                                 int nthreads)
{
    int nen = nen_of(p->etype), nd = 6 * nen;
    int status = 0;
    int64_t miss = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : status) reduction(+ : miss)
#endif
    for (int64_t e = 0; e < nelem; e++) {
        const int64_t *cn = conn + nen * e;
        double X[12], nr[12], Ke[24 * 24];
        uint8_t vl[4];
        int64_t dn[24];
        gather_X(xyz, nnodes, cn, nen, X);
        for (int a = 0; a < nen; a++) {
            int64_t node = cn[a] - 1;
            for (int c = 0; c < 3; c++) nr[3 * a + c] = normals[node + c * nnodes];
            vl[a] = valid[node];
            for (int k = 0; k < 6; k++) dn[6 * a + k] = dofnums[node + k * nnodes];
        }
        status |= orc_element_stiffness(p, e, X, nr, vl, Ke);
        for (int j = 0; j < nd; j++) {
            if (dn[j] < 1 || dn[j] > n) continue;
            const int64_t c0 = colptr[dn[j] - 1] - 1, c1 = colptr[dn[j]] - 1;
            for (int i = 0; i < nd; i++) {
                if (dn[i] < 1 || dn[i] > n) continue;
                int64_t lo = c0, hi = c1 - 1, at = -1;
                while (lo <= hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    if (rowval[mid] == dn[i]) { at = mid; break; }
                    if (rowval[mid] < dn[i]) lo = mid + 1; else hi = mid - 1;
                }
                if (at < 0) { miss++; continue; }
#ifdef _OPENMP
#pragma omp atomic
#endif
                vals[at] += Ke[IX(i, j, nd)];
                touched[at] = 1;
            }
        }
    }
    (void)nthreads;
    *missing = miss;
    return status;
}

/* Assembly of element matrices Ke (what 0, nelem x (6 nen)^2 column-major)
 * or of lumped masses tmrm (what 1, nelem x 2) in the given element order. */
static orc_result *assemble_from(int what, int mode, int nen, int64_t nnodes, int64_t nelem,
                                 const int64_t *conn, const int64_t *order, const int64_t *dofnums,
                                 int64_t n, const double *Ke, const double *tmrm)
{
    int nd = 6 * nen;
    orc_result *res = (orc_result *)calloc(1, sizeof(orc_result));
    res->n = n;
    if (mode == ORC_DIAG) {
        /* SysmatAssemblerSparseDiag: diagonal entries only */
        double *d = (double *)calloc(n > 0 ? n : 1, sizeof(double));
        for (int64_t r = 0; r < nelem; r++) {
            int64_t e = order ? order[r] : r;
            const int64_t *cn = conn + nen * e;
            for (int a = 0; a < nen; a++)
                for (int k = 0; k < 6; k++) {
                    int64_t dof = dofnums[(cn[a] - 1) + k * nnodes];
                    if (dof < 1 || dof > n) continue;
                    double v = what == 0 ? Ke[(int64_t)nd * nd * e + IX(6 * a + k, 6 * a + k, nd)]
                                         : tmrm[2 * e + (k < 3 ? 0 : 1)];
                    d[dof - 1] += v;
                }
        }
        res->nnz = n;
        res->colptr = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
        res->rowval = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
        res->nzval = d;
        for (int64_t i = 0; i <= n; i++) res->colptr[i] = i;
        for (int64_t i = 0; i < n; i++) res->rowval[i] = i;
    } else {
        int64_t cap = (int64_t)nelem * nd * nd;
        int64_t *I = (int64_t *)malloc(sizeof(int64_t) * (cap > 0 ? cap : 1));
        int64_t *J = (int64_t *)malloc(sizeof(int64_t) * (cap > 0 ? cap : 1));
        double *V = (double *)malloc(sizeof(double) * (cap > 0 ? cap : 1));
        int64_t m = 0;
        for (int64_t r = 0; r < nelem; r++) {
            int64_t e = order ? order[r] : r;
            const int64_t *cn = conn + nen * e;
            int64_t dn[24];
            for (int a = 0; a < nen; a++)
                for (int k = 0; k < 6; k++) dn[6 * a + k] = dofnums[(cn[a] - 1) + k * nnodes];
            for (int j = 0; j < nd; j++) {
                if (dn[j] < 1 || dn[j] > n) continue;
                for (int i = (mode == ORC_DROP_ZEROS ? j : 0); i < nd; i++) {
                    if (dn[i] < 1 || dn[i] > n) continue;
                    double v;
                    if (what == 0) v = Ke[(int64_t)nd * nd * e + IX(i, j, nd)];
                    else v = (i == j) ? tmrm[2 * e + ((i % 6) < 3 ? 0 : 1)] : 0.0;
                    I[m] = dn[i] - 1;
                    J[m] = dn[j] - 1;
                    V[m] = v;
                    m++;
                }
            }
        }
        int64_t *cp, *rv, nnz;
        double *nz;
        coo_to_csc(n, m, I, J, V, &cp, &rv, &nz, &nnz);
        free(I); free(J); free(V);
        if (mode == ORC_DROP_ZEROS) {
            int64_t *cp2, *rv2, nnz2;
            double *nz2;
            symm_complete(n, cp, rv, nz, &cp2, &rv2, &nz2, &nnz2);
            free(cp); free(rv); free(nz);
            cp = cp2; rv = rv2; nz = nz2; nnz = nnz2;
        }
        res->nnz = nnz;
        res->colptr = cp;
        res->rowval = rv;
        res->nzval = nz;
    }
    return res;
}

int orc_assemble(int what, int mode, int64_t nnodes, const double *xyz, int64_t nelem,
                 const int64_t *conn, const int64_t *order, const int64_t *dofnums, int64_t n,
                 const double *normals, const uint8_t *valid, const orc_params *p, int nthreads,
                 orc_result **out)
{
    int nen = nen_of(p->etype), nd = 6 * nen;
    double *Ke = NULL;
    double *tmrm = NULL;
    int status = 0;
    if (what == 0) {
        Ke = (double *)malloc(sizeof(double) * nd * nd * (nelem > 0 ? nelem : 1));
        status = orc_all_element_stiffness(nnodes, xyz, nelem, conn, normals, valid, p, nthreads, Ke);
        if (status) {
            free(Ke);
            return status;
        }
    } else {
        tmrm = (double *)malloc(sizeof(double) * 2 * (nelem > 0 ? nelem : 1));
        for (int64_t e = 0; e < nelem; e++) {
            double X[12];
            gather_X(xyz, nnodes, conn + nen * e, nen, X);
            orc_element_mass(p, e, X, tmrm + 2 * e, tmrm + 2 * e + 1);
        }
    }
    *out = assemble_from(what, mode, nen, nnodes, nelem, conn, order, dofnums, n, Ke, tmrm);
    free(Ke);
    free(tmrm);
    return 0;
}

int orc_assemble_elmats(int mode, int nen, int64_t nnodes, int64_t nelem, const int64_t *conn,
                        const int64_t *order, const int64_t *dofnums, int64_t n, const double *Ke,
                        orc_result **out)
{
    if (nen < 1 || nen > 4) return 1;
    *out = assemble_from(0, mode, nen, nnodes, nelem, conn, order, dofnums, n, Ke, NULL);
    return 0;
}

int64_t orc_result_nnz(const orc_result *r) { return r->nnz; }
int64_t orc_result_n(const orc_result *r) { return r->n; }
void orc_result_copy(const orc_result *r, int64_t *colptr, int64_t *rowval, double *nzval)
{
    for (int64_t i = 0; i <= r->n; i++) colptr[i] = r->colptr[i] + 1;
    for (int64_t k = 0; k < r->nnz; k++) {
        rowval[k] = r->rowval[k] + 1;
        nzval[k] = r->nzval[k];
    }
}
void orc_result_free(orc_result *r)
{
    if (!r) return;
    free(r->colptr);
    free(r->rowval);
    free(r->nzval);
    free(r);
}

/* ------------------------------------------------------------------ */
/* Explicit central difference, _cd_loop!,                              */
/* examples/shells/dynamics/homogeneous/explicit/plate_expl_examples.jl:61-94 */
/* ------------------------------------------------------------------ */
int orc_cd_steps(int64_t n, const int64_t *rowptr, const int64_t *colidx, const double *vals,
                 const double *invMC, const double *C, double dt, int64_t nsteps, double *U,
                 double *V, double *A, int nthreads)
{
    return orc_cd_steps_load(n, rowptr, colidx, vals, invMC, C, dt, nsteps, U, V, A, NULL, NULL, 0, 0,
                             nthreads);
}

/* the same loop with the external force of the example's force!(F, t) =
 * g(t) Fmag (plate_expl_examples.jl:202-209): mul[k] = g(k dt), the state at
 * step index step0 */
int orc_cd_steps_load(int64_t n, const int64_t *rowptr, const int64_t *colidx, const double *vals,
                      const double *invMC, const double *C, double dt, int64_t nsteps, double *U,
                      double *V, double *A, const double *Fmag, const double *mul, int64_t nmul,
                      int64_t step0, int nthreads)
{
    double dt2_2 = (dt * dt) / 2, dt_2 = dt / 2;
    double *F = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    (void)nthreads;
    for (int64_t step = 0; step < nsteps; step++) {
        const int64_t k = step0 + step + 1;
        const double g = (Fmag && k < nmul) ? mul[k] : 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < n; i++) U[i] += dt * V[i] + dt2_2 * A[i];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < n; i++) {
            double s = 0.0;
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) s += vals[k] * U[colidx[k]];
            double f = Fmag ? g * Fmag[i] : 0.0; /* external force F .= mul .* Fmag */
            f -= s + C[i] * (V[i] + dt_2 * A[i]);
            F[i] = f;
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < n; i++) {
            V[i] += dt_2 * A[i];
            A[i] = invMC[i] * F[i];
            V[i] += dt_2 * A[i];
        }
    }
    free(F);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Laminate: laminate_stiffnesses!, laminate_transverse_stiffness!,     */
/* laminate_inertia!, src/CompositeLayupModule.jl:246-330               */
/* ------------------------------------------------------------------ */
int orc_laminate(int nplies, const double *ply_Dps, const double *ply_Dts, const double *ply_t,
                 const double *ply_angle_deg, const double *ply_rho, double offset,
                 int shear_model, double tcf, double *A, double *B, double *D, double *H,
                 double *mass_density, double *moi_density)
{
    double lt = 0.0;
    for (int k = 0; k < nplies; k++) lt += ply_t[k];
    for (int i = 0; i < 9; i++) A[i] = B[i] = D[i] = 0.0;
    for (int i = 0; i < 4; i++) H[i] = 0.0;
    double zs = -lt / 2 - offset;
    for (int k = 0; k < nplies; k++) {
        double ze = zs + ply_t[k];
        double ang = ply_angle_deg[k] / 180 * M_PI;
        double m = cos(-ang), n = sin(-ang);
        double T[9];
        T[IX(0, 0, 3)] = m * m;    T[IX(0, 1, 3)] = n * n;    T[IX(0, 2, 3)] = 2 * (m * n);
        T[IX(1, 0, 3)] = n * n;    T[IX(1, 1, 3)] = m * m;    T[IX(1, 2, 3)] = -2 * (m * n);
        T[IX(2, 0, 3)] = -(m * n); T[IX(2, 1, 3)] = (m * n);  T[IX(2, 2, 3)] = m * m - n * n;
        double Dps[9];
        memcpy(Dps, ply_Dps + 9 * k, sizeof(Dps));
        qeqt(Dps, T, 3);
        for (int i = 0; i < 9; i++) {
            A[i] += (ze - zs) * Dps[i];
            B[i] += (ze * ze - zs * zs) / 2 * Dps[i];
            D[i] += (ze * ze * ze - zs * zs * zs) / 3 * Dps[i];
        }
        zs += ply_t[k];
    }
    zs = -lt / 2 - offset;
    for (int k = 0; k < nplies; k++) {
        double ze = zs + ply_t[k];
        double ang = ply_angle_deg[k] / 180 * M_PI;
        double m = cos(ang), n = sin(ang);
        double Tt[4] = {m, n, -n, m};
        double Dts[4];
        memcpy(Dts, ply_Dts + 4 * k, sizeof(Dts));
        qteq(Dts, Tt, 2);
        for (int i = 0; i < 4; i++) {
            if (shear_model == 0)
                H[i] += 5.0 / 4 * (ze - zs - 4.0 / 3 * (ze * ze * ze - zs * zs * zs) / (lt * lt)) * Dts[i];
            else
                H[i] += tcf * (ze - zs) * Dts[i];
        }
        zs += ply_t[k];
    }
    double md = 0.0, mi = 0.0;
    zs = -lt / 2 - offset;
    for (int k = 0; k < nplies; k++) {
        double ze = zs + ply_t[k];
        double rho = ply_rho ? ply_rho[k] : 0.0;
        md += (ze - zs) * rho;
        mi += (ze * ze * ze - zs * zs * zs) * rho / 3;
        zs += ply_t[k];
    }
    *mass_density = md;
    *moi_density = mi;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Stress resultants at the integration points of the homogeneous      */
/* shells: inspectintegpoints, src/FEMMShellT3FFModule.jl:850-962 (one */
/* point per element, the centroid) and src/FEMMShellQ4RSModule.jl:    */
/* 1061-1170 (the four Gauss points)                                   */
/* ------------------------------------------------------------------ */

/* the 2x2 tensor [v0 v2; v2 v1] (or the vector (v0, v1) of the shear
 * forces) seen in the output csys: o2 = [m n; -n m] from
 * Layup2ElementAngle(E_G, csmat); mo = o2' m o2, fo = o2' f */
static void resultant_out(const double *E, const double *cs, int quant, const double *v, double *out)
{
    double m, n;
    layup_angle(E, cs, &m, &n);
    double o[4];
    o[IX(0, 0, 2)] = m; o[IX(0, 1, 2)] = n;
    o[IX(1, 0, 2)] = -n; o[IX(1, 1, 2)] = m;
    if (quant == ORC_RES_SHEAR) {
        out[0] = o[IX(0, 0, 2)] * v[0] + o[IX(1, 0, 2)] * v[1];
        out[1] = o[IX(0, 1, 2)] * v[0] + o[IX(1, 1, 2)] * v[1];
        out[2] = 0.0;
        return;
    }
    double M[4], t[4], R[4];
    M[IX(0, 0, 2)] = v[0]; M[IX(0, 1, 2)] = v[2];
    M[IX(1, 0, 2)] = v[2]; M[IX(1, 1, 2)] = v[1];
    for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) t[IX(i, j, 2)] = o[IX(0, i, 2)] * M[IX(0, j, 2)] + o[IX(1, i, 2)] * M[IX(1, j, 2)];
    for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) R[IX(i, j, 2)] = t[IX(i, 0, 2)] * o[IX(0, j, 2)] + t[IX(i, 1, 2)] * o[IX(1, j, 2)];
    out[0] = R[IX(0, 0, 2)];
    out[1] = R[IX(1, 1, 2)];
    out[2] = R[IX(0, 1, 2)];
}

static void matvec(const double *A, int r, int c, const double *x, double *y)
{
    for (int i = 0; i < r; i++) {
        double s = 0.0;
        for (int k = 0; k < c; k++) s += A[IX(i, k, r)] * x[k];
        y[i] = s;
    }
}

/* material times strain: moment t^3/12 Dps kurv, membrane t Dps strn,
 * shear t stab (5/6 Dt) shr */
static void resultant_material(const orc_params *p, int quant, double t, double stab, const double *s,
                               double *v)
{
    if (quant == ORC_RES_SHEAR) {
        double Dt5[4];
        for (int i = 0; i < 4; i++) Dt5[i] = p->Dt[i] * (5.0 / 6.0);
        double f = t * stab;
        for (int i = 0; i < 2; i++) v[i] = f * (Dt5[IX(i, 0, 2)] * s[0] + Dt5[IX(i, 1, 2)] * s[1]);
        v[2] = 0.0;
        return;
    }
    double f = quant == ORC_RES_MOMENT ? (t * t * t) / 12 : t;
    for (int i = 0; i < 3; i++)
        v[i] = f * (p->Dps[IX(i, 0, 3)] * s[0] + p->Dps[IX(i, 1, 3)] * s[1] + p->Dps[IX(i, 2, 3)] * s[2]);
}

static void t3_resultant(const orc_params *p, int64_t e, const double *X, const double *nrm,
                         const uint8_t *valid, const double *ed, int quant, const double *cs, double *out)
{
    const int n = 18;
    double J0[6], E[9], ee[6], g[6];
    for (int j = 0; j < 3; j++) {
        J0[IX(j, 0, 3)] = X[3 * 1 + j] - X[3 * 0 + j];
        J0[IX(j, 1, 3)] = X[3 * 2 + j] - X[3 * 0 + j];
    }
    e_g(E, J0);
    ee[IX(0, 0, 3)] = ee[IX(0, 1, 3)] = 0.0;
    ee[IX(1, 0, 3)] = J0[0] * E[0] + J0[1] * E[1] + J0[2] * E[2];
    ee[IX(1, 1, 3)] = J0[0] * E[3] + J0[1] * E[4] + J0[2] * E[5];
    ee[IX(2, 0, 3)] = J0[3] * E[0] + J0[4] * E[1] + J0[5] * E[2];
    ee[IX(2, 1, 3)] = J0[3] * E[3] + J0[4] * E[4] + J0[5] * E[5];
    double a = ee[IX(1, 0, 3)] - ee[IX(0, 0, 3)], b = ee[IX(1, 1, 3)] - ee[IX(0, 1, 3)];
    double c = ee[IX(2, 0, 3)] - ee[IX(0, 0, 3)], d = ee[IX(2, 1, 3)] - ee[IX(0, 1, 3)];
    double J = a * d - b * c;
    g[IX(0, 0, 3)] = (b - d) / J; g[IX(1, 0, 3)] = d / J; g[IX(2, 0, 3)] = -b / J;
    g[IX(0, 1, 3)] = (c - a) / J; g[IX(1, 1, 3)] = -c / J; g[IX(2, 1, 3)] = a / J;
    double Ae = J / 2;
    double t;
    elem_thickness(p, e, &t);
    /* global -> nodal -> element displacements */
    double AEs[27], T[18 * 18], edn[18], ede[18];
    uint8_t nv[3];
    nodal_triads(AEs, nv, E, nrm, valid, 3);
    transfmat_g_to_a(T, AEs, E, 3);
    matvec(T, n, n, ed, edn);
    transfmat_a_to_e(T, AEs, g, 3);
    matvec(T, n, n, edn, ede);
    double s[3] = {0, 0, 0}, v[3];
    if (quant == ORC_RES_MOMENT || quant == ORC_RES_MEMBRANE) {
        double B[3 * 18] = {0};
        for (int i = 0; i < 3; i++) {
            if (quant == ORC_RES_MEMBRANE) {
                B[IX(0, 6 * i + 0, 3)] = g[IX(i, 0, 3)];
                B[IX(1, 6 * i + 1, 3)] = g[IX(i, 1, 3)];
                B[IX(2, 6 * i + 0, 3)] = g[IX(i, 1, 3)];
                B[IX(2, 6 * i + 1, 3)] = g[IX(i, 0, 3)];
            } else {
                B[IX(0, 6 * i + 4, 3)] = g[IX(i, 0, 3)];
                B[IX(1, 6 * i + 3, 3)] = -g[IX(i, 1, 3)];
                B[IX(2, 6 * i + 3, 3)] = -g[IX(i, 0, 3)];
                B[IX(2, 6 * i + 4, 3)] = g[IX(i, 1, 3)];
            }
        }
        matvec(B, 3, n, ede, s);
        resultant_material(p, quant, t, 0.0, s, v);
    } else {
        /* _Bsmat!: the DSG rows averaged over the three node orderings */
        double Bs[2 * 18] = {0};
        add_bsmat_o(Bs, ee, Ae, 0, 1, 2);
        add_bsmat_o(Bs, ee, Ae, 1, 2, 0);
        add_bsmat_o(Bs, ee, Ae, 2, 0, 1);
        for (int i = 0; i < 36; i++) Bs[i] *= (1.0 / 3);
        matvec(Bs, 2, n, ede, s);
        resultant_material(p, quant, t, stab_fun(t, sqrt(2 * Ae), p->stab_c), s, v);
    }
    /* default mcsys: isoparametric! = _e_g!(J0), the element frame */
    resultant_out(E, cs ? cs : E, quant, v, out);
}

static void q4_resultants(const orc_params *p, int64_t e, const double *X, const double *nrm,
                          const uint8_t *valid, const double *ed, int quant, const double *cs,
                          int64_t cs_stride, double *out /* 4 x 3 */)
{
    const int n = 24;
    double t;
    elem_thickness(p, e, &t);
    double h = q4_diameter(X);
    double *T = (double *)malloc(sizeof(double) * 3 * n * n);
    double *Tae = T + n * n, *Tga = T + 2 * n * n;
    for (int j = 0; j < 4; j++) {
        double xi, eta, N[4], gp[8], J[6], E[9], ee[8], g[8];
        q4_point(j, &xi, &eta);
        q4_basis(xi, eta, N, gp);
        q4_jac(X, gp, J);
        e_g(E, J);
        double cen[3] = {0, 0, 0};
        for (int a = 0; a < 4; a++)
            for (int k = 0; k < 3; k++) cen[k] += X[3 * a + k];
        for (int k = 0; k < 3; k++) cen[k] /= 4;
        for (int a = 0; a < 4; a++)
            for (int k = 0; k < 2; k++) {
                double dd = 0.0;
                for (int m = 0; m < 3; m++) dd += (X[3 * a + m] - cen[m]) * E[IX(m, k, 3)];
                ee[IX(a, k, 4)] = dd;
            }
        double G11 = J[0] * J[0] + J[1] * J[1] + J[2] * J[2];
        double G12 = J[0] * J[3] + J[1] * J[4] + J[2] * J[5];
        double G22 = J[3] * J[3] + J[4] * J[4] + J[5] * J[5];
        double detG = G11 * G22 - G12 * G12;
        double i11 = G22 / detG, i12 = -G12 / detG, i22 = G11 / detG;
        for (int a = 0; a < 4; a++) {
            double t1 = i11 * gp[IX(a, 0, 4)] + i12 * gp[IX(a, 1, 4)];
            double t2 = i12 * gp[IX(a, 0, 4)] + i22 * gp[IX(a, 1, 4)];
            double vv[3];
            for (int c = 0; c < 3; c++) vv[c] = J[IX(c, 0, 3)] * t1 + J[IX(c, 1, 3)] * t2;
            g[IX(a, 0, 4)] = E[0] * vv[0] + E[1] * vv[1] + E[2] * vv[2];
            g[IX(a, 1, 4)] = E[3] * vv[0] + E[4] * vv[1] + E[5] * vv[2];
        }
        double AEs[36];
        uint8_t nv[4];
        nodal_triads(AEs, nv, E, nrm, valid, 4);
        transfmat_g_to_a(Tga, AEs, E, 4);
        transfmat_a_to_e(Tae, AEs, g, 4);
        matmul_rn(Tae, n, n, Tga, n, T);
        double ede[24];
        matvec(T, n, n, ed, ede);
        double s[3] = {0, 0, 0}, v[3];
        if (quant == ORC_RES_MOMENT || quant == ORC_RES_MEMBRANE) {
            double B[3 * 24] = {0};
            for (int i = 0; i < 4; i++) {
                int off = 6 * i;
                if (quant == ORC_RES_MEMBRANE) {
                    B[IX(0, off + 0, 3)] = g[IX(i, 0, 4)];
                    B[IX(1, off + 1, 3)] = g[IX(i, 1, 4)];
                    B[IX(2, off + 0, 3)] = g[IX(i, 1, 4)];
                    B[IX(2, off + 1, 3)] = g[IX(i, 0, 4)];
                } else {
                    B[IX(0, off + 4, 3)] = g[IX(i, 0, 4)];
                    B[IX(1, off + 3, 3)] = -g[IX(i, 1, 4)];
                    B[IX(2, off + 3, 3)] = -g[IX(i, 0, 4)];
                    B[IX(2, off + 4, 3)] = g[IX(i, 1, 4)];
                }
            }
            matvec(B, 3, n, ede, s);
            resultant_material(p, quant, t, 0.0, s, v);
        } else {
            double Bs[2 * 24];
            q4_bs_elem(Bs, ee, xi, eta);
            matvec(Bs, 2, n, ede, s);
            resultant_material(p, quant, t, stab_fun(t, h, p->stab_c), s, v);
        }
        /* default mcsys: _isoparametric! = _e_g!(J), the frame at the point */
        resultant_out(E, cs ? cs + cs_stride * j : E, quant, v, out + 3 * j);
    }
    free(T);
}

int orc_resultants(int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                   const double *normals, const uint8_t *valid, const orc_params *p,
                   const double *u, int quant, const double *cs, int64_t ncs, double *out)
{
    if (p->etype != ORC_T3FF && p->etype != ORC_Q4RS) return 1;
    if (quant < ORC_RES_MOMENT || quant > ORC_RES_MEMBRANE) return 2;
    const int nen = nen_of(p->etype), npt = nen == 3 ? 1 : 4;
    if (ncs != 0 && ncs != 1 && ncs != nelem * npt) return 3;
    for (int64_t e = 0; e < nelem; e++) {
        const int64_t *cn = conn + nen * e;
        double X[12], nrm[12], ed[24];
        uint8_t vl[4];
        gather_X(xyz, nnodes, cn, nen, X);
        for (int k = 0; k < nen; k++) {
            int64_t nd = cn[k] - 1;
            for (int c = 0; c < 3; c++) nrm[3 * k + c] = normals[nd + c * nnodes];
            vl[k] = valid[nd];
            for (int c = 0; c < 6; c++) ed[6 * k + c] = u[nd + c * nnodes];
        }
        const double *c0 = ncs == 0 ? NULL : (ncs == 1 ? cs : cs + 9 * npt * e);
        const int64_t cst = ncs == 1 ? 0 : 9;
        if (nen == 3)
            t3_resultant(p, e, X, nrm, vl, ed, quant, c0, out + 3 * e);
        else
            q4_resultants(p, e, X, nrm, vl, ed, quant, c0, cst, out + 12 * e);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* distributed surface loads: FinEtools 8.2.5 distribloads(FEMMBase,   */
/* geom, P, fi::ForceIntensity, m) on the shell element sets           */
/* (plate_expl_examples.jl:196-199, test/test_shell_statics.jl:84-86)  */
/* ------------------------------------------------------------------ */

/* integration rule on the parent element: TriRule(npts) for triangles
 * (1: centroid; 3: the degree-2 interior points; 6: Dunavant's degree-4
 * rule, orbits (1-2a, a) and permutations), GaussRule(2, order) for
 * quadrilaterals (xi the outer index), GaussRule(1, order) for the line
 * element; param (npts x 2), weights */
static int surface_rule(int nen, int rule, double *pc, double *w)
{
    if (nen == 3) {
        if (rule == 1) {
            pc[0] = pc[1] = 1.0 / 3.0;
            w[0] = 0.5;
            return 1;
        }
        if (rule == 3) {
            const double P[3][2] = {{2.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {1.0 / 6.0, 1.0 / 6.0}};
            for (int j = 0; j < 3; j++) {
                pc[2 * j] = P[j][0];
                pc[2 * j + 1] = P[j][1];
                w[j] = 1.0 / 6.0;
            }
            return 3;
        }
        if (rule == 6) {
            const double a[2] = {0.445948490915965, 0.091576213509771};
            const double wt[2] = {0.223381589678011, 0.109951743655322};
            for (int o = 0; o < 2; o++) {
                const double b = 1.0 - 2.0 * a[o];
                const double P[3][2] = {{b, a[o]}, {a[o], b}, {a[o], a[o]}};
                for (int j = 0; j < 3; j++) {
                    pc[2 * (3 * o + j)] = P[j][0];
                    pc[2 * (3 * o + j) + 1] = P[j][1];
                    w[3 * o + j] = wt[o] / 2.0;
                }
            }
            return 6;
        }
        return 0;
    }
    double g[3], gw[3];
    if (nen != 2 && nen != 4) return 0;
    if (rule == 1) {
        g[0] = 0.0;
        gw[0] = 2.0;
    } else if (rule == 2) {
        g[0] = -1.0 / sqrt(3.0);
        g[1] = 1.0 / sqrt(3.0);
        gw[0] = gw[1] = 1.0;
    } else if (rule == 3) {
        g[0] = -sqrt(0.6);
        g[1] = 0.0;
        g[2] = sqrt(0.6);
        gw[0] = gw[2] = 5.0 / 9.0;
        gw[1] = 8.0 / 9.0;
    } else {
        return 0;
    }
    if (nen == 2) {
        /* GaussRule(1, order) on the line element, eta unused */
        for (int i = 0; i < rule; i++) {
            pc[2 * i] = g[i];
            pc[2 * i + 1] = 0.0;
            w[i] = gw[i];
        }
        return rule;
    }
    int r = 0;
    for (int i = 0; i < rule; i++)
        for (int j = 0; j < rule; j++, r++) {
            pc[2 * r] = g[i];
            pc[2 * r + 1] = g[j];
            w[r] = gw[i] * gw[j];
        }
    return r;
}

/* bfunparam / bfundparams of FESetL2, FESetT3 and FESetQ4: N (nen), gradN
 * (nen x 2, column-major; the second column zero for the line element) */
static void surface_basis(int nen, double xi, double eta, double *N, double *gN)
{
    if (nen == 2) {
        N[0] = 0.5 * (1.0 - xi);
        N[1] = 0.5 * (1.0 + xi);
        const double g[4] = {-0.5, 0.5, 0.0, 0.0};
        memcpy(gN, g, sizeof g);
        return;
    }
    if (nen == 3) {
        N[0] = 1.0 - xi - eta;
        N[1] = xi;
        N[2] = eta;
        const double g[6] = {-1.0, 1.0, 0.0, -1.0, 0.0, 1.0};
        memcpy(gN, g, sizeof g);
        return;
    }
    const double s[4] = {-1.0, 1.0, 1.0, -1.0}, t[4] = {-1.0, -1.0, 1.0, 1.0};
    for (int a = 0; a < 4; a++) {
        N[a] = 0.25 * (1.0 + s[a] * xi) * (1.0 + t[a] * eta);
        gN[a] = 0.25 * s[a] * (1.0 + t[a] * eta);
        gN[4 + a] = 0.25 * t[a] * (1.0 + s[a] * xi);
    }
}

/* locjac!: loc = N' X, J = X' gradN (3 x 2, column-major), X nen x 3 row per node */
static void surface_locjac(int nen, const double *X, const double *N, const double *gN, double *loc, double *J)
{
    for (int i = 0; i < 3; i++) {
        double l = 0.0, j1 = 0.0, j2 = 0.0;
        for (int a = 0; a < nen; a++) {
            l += N[a] * X[3 * a + i];
            j1 += X[3 * a + i] * gN[a];
            j2 += X[3 * a + i] * gN[nen + a];
        }
        loc[i] = l;
        J[i] = j1;
        J[3 + i] = j2;
    }
}

int orc_integration_points(int nen, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                           int rule, double *out)
{
    double pc[18], w[9], N[4], gN[8];
    const int np = surface_rule(nen, rule, pc, w);
    if (!np) return 1;
    for (int64_t e = 0; e < nelem; e++) {
        double X[12];
        gather_X(xyz, nnodes, conn + nen * e, nen, X);
        for (int j = 0; j < np; j++) {
            double *o = out + 9 * (e * np + j);
            surface_basis(nen, pc[2 * j], pc[2 * j + 1], N, gN);
            surface_locjac(nen, X, N, gN, o, o + 3);
        }
    }
    return 0;
}

int orc_distribloads(int nen, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                     const int64_t *dofnums, int rule, int m, const double *force, int64_t nforce, int64_t n,
                     double *F)
{
    double pc[18], w[9], N[4], gN[8];
    const int np = surface_rule(nen, rule, pc, w);
    if (!np) return 1;
    if (m < (nen == 2 ? 1 : 2) || m > 3) return 2;
    if (nforce != 1 && nforce != nelem && nforce != nelem * np) return 3;
    for (int64_t d = 0; d < n; d++) F[d] = 0.0;
    for (int64_t e = 0; e < nelem; e++) {
        double X[12], Fe[24], loc[3], J[6];
        gather_X(xyz, nnodes, conn + nen * e, nen, X);
        memset(Fe, 0, sizeof Fe);
        for (int j = 0; j < np; j++) {
            surface_basis(nen, pc[2 * j], pc[2 * j + 1], N, gN);
            surface_locjac(nen, X, N, gN, loc, J);
            /* Jacobiancurve |x,xi| of the line element, Jacobiansurface |x,xi x x,eta|
             * of the surface elements; the higher manifold dimensions multiply by
             * the other dimension 1 (FEMMBase's default) */
            double Jac;
            if (nen == 2) {
                Jac = sqrt(J[0] * J[0] + J[1] * J[1] + J[2] * J[2]);
            } else {
                const double a1 = J[1] * J[5] - J[2] * J[4];
                const double a2 = J[2] * J[3] - J[0] * J[5];
                const double a3 = J[0] * J[4] - J[1] * J[3];
                Jac = sqrt(a1 * a1 + a2 * a2 + a3 * a3);
            }
            const double factor = Jac * w[j];
            const double *f = nforce == 1 ? force : (nforce == nelem ? force + 6 * e : force + 6 * (e * np + j));
            for (int a = 0; a < nen; a++) {
                const double Nf = N[a] * factor;
                for (int k = 0; k < 6; k++) Fe[6 * a + k] += Nf * f[k];
            }
        }
        /* SysvecAssembler: F[dof] += Fe in element order; dofs above n dropped */
        for (int a = 0; a < nen; a++) {
            const int64_t nd = conn[nen * e + a] - 1;
            for (int k = 0; k < 6; k++) {
                const int64_t d = dofnums[nd + k * nnodes];
                if (d >= 1 && d <= n) F[d - 1] += Fe[6 * a + k];
            }
        }
    }
    return 0;
}

// Host-side preparation of the per-call material constants.
#pragma once
#include <math.h>
#include <string.h>

#include "../../include/flexshell.h"
#include "fs_elem_math.cuh"

namespace fs {

// Cholesky factor of a symmetric positive semi-definite n x n matrix
// (column-major), lower triangle packed row by row.  A zero pivot is
// accepted only when the rest of its column is zero (a material with a
// vanishing stiffness component).  Returns 0 or 1 (not semi-definite).
inline int chol_packed(const double *A, int n, double *L)
{
    double W[6][6];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) W[i][j] = A[i + j * n];
    double scale = 0.0;
    for (int i = 0; i < n; i++) scale = fmax(scale, fabs(W[i][i]));
    for (int j = 0; j < n; j++) {
        double d = W[j][j];
        for (int k = 0; k < j; k++) d -= L[lp(j, k)] * L[lp(j, k)];
        if (d < -1e-12 * scale) return 1;
        double ljj = d > 1e-300 * (scale + 1e-300) ? sqrt(d) : 0.0;
        L[lp(j, j)] = ljj;
        for (int i = j + 1; i < n; i++) {
            double s = W[i][j];
            for (int k = 0; k < j; k++) s -= L[lp(i, k)] * L[lp(j, k)];
            if (ljj == 0.0) {
                if (fabs(s) > 1e-12 * scale) return 1;
                L[lp(i, j)] = 0.0;
            } else {
                L[lp(i, j)] = s / ljj;
            }
        }
    }
    return 0;
}

inline int prepare_matconst(const fs_shell_params &p, MatConst &mc)
{
    memset(&mc, 0, sizeof(mc));
    double Dps[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) Dps[i + 3 * j] = 0.5 * (p.Dps[i + 3 * j] + p.Dps[j + 3 * i]);
    if (chol_packed(Dps, 3, mc.Lps)) return 1;
    double Dt[4];
    for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) Dt[i + 2 * j] = (5.0 / 6.0) * 0.5 * (p.Dt[i + 2 * j] + p.Dt[j + 2 * i]);
    if (chol_packed(Dt, 2, mc.Lt)) return 1;
    mc.stab_c = p.stab_c;
    mc.drill_scale = p.drilling_stiffness_scale;
    mc.drill_scale6 = p.drilling_stiffness_scale / 6.0;
    mc.rho = p.rho;
    for (int i = 0; i < 6; i++) mc.Lpsf[i] = (float)mc.Lps[i];
    for (int i = 0; i < 3; i++) mc.Ltf[i] = (float)mc.Lt[i];
    mc.stab_cf = (float)mc.stab_c;
    for (int i = 0; i < 9; i++) mc.Dps[i] = Dps[i];
    for (int i = 0; i < 4; i++) mc.Dt5[i] = Dt[i];
    return 0;
}

inline int prepare_group(const fs_layup_group &g, GroupConst &gc)
{
    memset(&gc, 0, sizeof(gc));
    double ABD[36];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double a = 0.5 * (g.A[i + 3 * j] + g.A[j + 3 * i]);
            double b = 0.5 * (g.B[i + 3 * j] + g.B[j + 3 * i]);
            double d = 0.5 * (g.D[i + 3 * j] + g.D[j + 3 * i]);
            ABD[i + 6 * j] = a;
            ABD[(i + 3) + 6 * (j + 3)] = d;
            ABD[(i + 3) + 6 * j] = b;
            ABD[i + 6 * (j + 3)] = b;
        }
    if (chol_packed(ABD, 6, gc.L6)) return 1;
    double H[4];
    for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) H[i + 2 * j] = 0.5 * (g.H[i + 2 * j] + g.H[j + 2 * i]);
    if (chol_packed(H, 2, gc.LH)) return 1;
    memcpy(gc.csmat, g.csmat, sizeof(gc.csmat));
    gc.thickness = g.thickness;
    gc.mass = g.mass_density;
    gc.moi = g.moi_density;
    for (int i = 0; i < 21; i++) gc.L6f[i] = (float)gc.L6[i];
    for (int i = 0; i < 3; i++) gc.LHf[i] = (float)gc.LH[i];
    return 0;
}

}  // namespace fs

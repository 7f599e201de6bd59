/*
 * CPU oracle for the co-rotational beam (FEMMCorotBeam) element loops.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of
 * src/FEMMCorotBeamModule.jl (FinEtoolsFlexStructures.jl 3.6.4) and of
 * initial_local_frame! (src/FESetL2BeamModule.jl:108-127), used as the
 * checker of the CUDA beam kernels.  The product never links it.
 *
 * It keeps the reference's own dense steps: the 6x12 natural-to-Cartesian
 * matrix aN, SM = aN' DN aN, and the 12x12 congruence Te SM Te' with the
 * block-diagonal Te = diag(Ft, Ft, Ft, Ft).
 *
 * Conventions: element nodal data are rows per node (x0, u: 2 x 3 stored
 * node-major, x0[3*a + c]); rotation matrices are column-major 3 x 3, the
 * layout of R1I[:] .= Rfield1.values[node, :]; element matrices are
 * column-major 12 x 12.
 */
#include <math.h>
#include <string.h>

#include "corotbeam_oracle.h"

#define M3(i, j) ((i) + 3 * (j))
#define M12(i, j) ((i) + 12 * (j))
#define M6(i, j) ((i) + 6 * (j))

/* C = A B, 3 x 3 column-major */
static void mm3(double *C, const double *A, const double *B)
{
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += A[M3(i, k)] * B[M3(k, j)];
            C[M3(i, j)] = s;
        }
}

/* C = A' B, 3 x 3 column-major */
static void mtm3(double *C, const double *A, const double *B)
{
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += A[M3(k, i)] * B[M3(k, j)];
            C[M3(i, j)] = s;
        }
}

static double norm3(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

/* column 3 = column 1 x v (normalised), column 2 = column 3 x column 1:
 * the explicit skewmat products of src/FESetL2BeamModule.jl:112-125 and
 * src/FEMMCorotBeamModule.jl:161-180 */
static void complete_frame(double *F, const double *v)
{
    F[M3(0, 2)] = -F[M3(2, 0)] * v[1] + F[M3(1, 0)] * v[2];
    F[M3(1, 2)] = F[M3(2, 0)] * v[0] - F[M3(0, 0)] * v[2];
    F[M3(2, 2)] = -F[M3(1, 0)] * v[0] + F[M3(0, 0)] * v[1];
    double n3 = norm3(F + 6);
    for (int i = 0; i < 3; i++) F[M3(i, 2)] /= n3;
    F[M3(0, 1)] = -F[M3(2, 2)] * F[M3(1, 0)] + F[M3(1, 2)] * F[M3(2, 0)];
    F[M3(1, 1)] = F[M3(2, 2)] * F[M3(0, 0)] - F[M3(0, 2)] * F[M3(2, 0)];
    F[M3(2, 1)] = -F[M3(1, 2)] * F[M3(0, 0)] + F[M3(0, 2)] * F[M3(1, 0)];
}

/* initial_local_frame!, src/FESetL2BeamModule.jl:108-127 */
static double initial_frame(double *F0, const double *x0, const double *x1x2)
{
    for (int c = 0; c < 3; c++) F0[M3(c, 0)] = x0[3 + c] - x0[c];
    double L0 = norm3(F0);
    for (int c = 0; c < 3; c++) F0[M3(c, 0)] /= L0;
    complete_frame(F0, x1x2);
    return L0;
}

/* local_frame_and_def!, src/FEMMCorotBeamModule.jl:208-243 (with
 * current_local_frame! :155-181) */
double orc_beam_frame(const double *x0, const double *xt, const double *x1x2, const double *RI,
                      const double *RJ, double *Ft, double *dN)
{
    double F0[9], FtI[9], FtJ[9], LI[9], LJ[9];
    double L0 = initial_frame(F0, x0, x1x2);
    mm3(FtI, RI, F0);
    mm3(FtJ, RJ, F0);
    for (int c = 0; c < 3; c++) Ft[M3(c, 0)] = xt[3 + c] - xt[c];
    double Lt = norm3(Ft);
    for (int c = 0; c < 3; c++) Ft[M3(c, 0)] /= Lt;
    double v[3];
    for (int c = 0; c < 3; c++) v[c] = FtI[M3(c, 1)] + FtJ[M3(c, 1)];
    complete_frame(Ft, v);
    mtm3(LI, Ft, FtI);
    mtm3(LJ, Ft, FtJ);
    dN[0] = Lt - L0;
    dN[5] = (LJ[M3(2, 1)] / LJ[M3(1, 1)] - LI[M3(2, 1)] / LI[M3(1, 1)] - LJ[M3(1, 2)] / LJ[M3(2, 2)] +
             LI[M3(1, 2)] / LI[M3(2, 2)]) /
            2;
    double TH2I = -LI[M3(2, 0)] / LI[M3(0, 0)];
    double TH2J = -LJ[M3(2, 0)] / LJ[M3(0, 0)];
    double TH3I = LI[M3(1, 0)] / LI[M3(0, 0)];
    double TH3J = LJ[M3(1, 0)] / LJ[M3(0, 0)];
    dN[1] = TH3I - TH3J;
    dN[2] = TH3I + TH3J;
    dN[3] = -TH2I + TH2J;
    dN[4] = -TH2I - TH2J;
    return Lt;
}

/* local_cartesian_to_natural!, src/FEMMCorotBeamModule.jl:265-289 (6 x 12) */
static void cartesian_to_natural(double *aN, double L)
{
    memset(aN, 0, sizeof(double) * 72);
    aN[M6(0, 0)] = -1;
    aN[M6(0, 6)] = +1;
    aN[M6(1, 5)] = +1;
    aN[M6(1, 11)] = -1;
    aN[M6(2, 1)] = 2 / L;
    aN[M6(2, 5)] = +1;
    aN[M6(2, 7)] = -2 / L;
    aN[M6(2, 11)] = +1;
    aN[M6(3, 4)] = -1;
    aN[M6(3, 10)] = +1;
    aN[M6(4, 2)] = 2 / L;
    aN[M6(4, 4)] = -1;
    aN[M6(4, 8)] = -2 / L;
    aN[M6(4, 10)] = -1;
    aN[M6(5, 3)] = -1;
    aN[M6(5, 9)] = +1;
}

/* natural_stiffness!, src/FEMMCorotBeamModule.jl:729-779: Bernoulli when
 * either shear area is infinite, else Timoshenko; diagonal 6 x 6 */
static void natural_stiffness(double *DN, double E, double G, const double *s, double L)
{
    const double A = s[0], I2 = s[2], I3 = s[3], J = s[4], A2s = s[5], A3s = s[6];
    DN[0] = E * A / L;
    DN[1] = E * I3 / L;
    DN[3] = E * I2 / L;
    DN[5] = G * J / L;
    if (isinf(A2s) || isinf(A3s)) {
        DN[2] = 3 * E * I3 / L;
        DN[4] = 3 * E * I2 / L;
    } else {
        double Phi3 = 12 * E * I3 / (G * A2s * L * L);
        double Phi2 = 12 * E * I2 / (G * A3s * L * L);
        DN[2] = 3 * E * I3 / L / (1 + Phi3);
        DN[4] = 3 * E * I2 / L / (1 + Phi2);
    }
}

/* elmat <- Te elmat Te' with Te = diag(Ft, Ft, Ft, Ft) (_transfmat!, :135-138,
 * and the two mul! of every loop) */
static void rotate12(double *K, const double *Ft)
{
    double Te[144], T1[144];
    memset(Te, 0, sizeof(Te));
    for (int b = 0; b < 4; b++)
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) Te[M12(3 * b + i, 3 * b + j)] = Ft[M3(i, j)];
    /* T1 = K Te' */
    for (int j = 0; j < 12; j++)
        for (int i = 0; i < 12; i++) {
            double s = 0.0;
            for (int k = 0; k < 12; k++) s += K[M12(i, k)] * Te[M12(j, k)];
            T1[M12(i, j)] = s;
        }
    /* K = Te T1 */
    for (int j = 0; j < 12; j++)
        for (int i = 0; i < 12; i++) {
            double s = 0.0;
            for (int k = 0; k < 12; k++) s += Te[M12(i, k)] * T1[M12(k, j)];
            K[M12(i, j)] = s;
        }
}

/* complete_lt!: copy the upper triangle into the lower one */
static void complete_lt(double *K)
{
    for (int j = 0; j < 12; j++)
        for (int i = j + 1; i < 12; i++) K[M12(i, j)] = K[M12(j, i)];
}

/* local_geometric_stiffness!, src/FEMMCorotBeamModule.jl:321-382 (upper blocks
 * written, then mirrored) */
static void local_geometric_stiffness(double *SM, const double *PN, double L)
{
    const double N = PN[0], S_2 = -2 * PN[2] / L, S_3 = -2 * PN[4] / L, M_1 = PN[5];
    const double M_2I = PN[3] + PN[4], M_2J = PN[3] - PN[4];
    const double M_3I = -(PN[1] + PN[2]), M_3J = -(PN[1] - PN[2]);
    memset(SM, 0, sizeof(double) * 144);
#define S(i, j, v) SM[M12((i) - 1, (j) - 1)] = (v)
    /* [1:3, 1:3] */
    S(1, 2, -S_2 / L); S(1, 3, -S_3 / L);
    S(2, 1, -S_2 / L); S(2, 2, N / L);
    S(3, 1, -S_3 / L); S(3, 3, N / L);
    /* [1:3, 4:6] */
    S(2, 4, -M_2I / L); S(2, 5, M_1 / L);
    S(3, 4, -M_3I / L); S(3, 6, M_1 / L);
    /* [1:3, 7:9] */
    S(1, 8, S_2 / L); S(1, 9, S_3 / L);
    S(2, 7, S_2 / L); S(2, 8, -N / L);
    S(3, 7, S_3 / L); S(3, 9, -N / L);
    /* [1:3, 10:12] */
    S(2, 10, M_2J / L); S(2, 11, -M_1 / L);
    S(3, 10, M_3J / L); S(3, 12, -M_1 / L);
    /* [4:6, 4:6] */
    S(4, 5, M_3I / 2); S(4, 6, -M_2I / 2);
    S(5, 4, M_3I / 2);
    S(6, 4, -M_2I / 2);
    /* [4:6, 7:9] */
    S(4, 8, M_2I / L); S(4, 9, M_3I / L);
    S(5, 8, -M_1 / L);
    S(6, 9, -M_1 / L);
    /* [4:6, 10:12] */
    S(5, 12, M_1 / 2);
    S(6, 11, -M_1 / 2);
    /* [7:9, 7:9] */
    S(7, 8, -S_2 / L); S(7, 9, -S_3 / L);
    S(8, 7, -S_2 / L); S(8, 8, N / L);
    S(9, 7, -S_3 / L); S(9, 9, N / L);
    /* [7:9, 10:12] */
    S(8, 10, -M_2J / L); S(8, 11, M_1 / L);
    S(9, 10, -M_3J / L); S(9, 12, M_1 / L);
    /* [10:12, 10:12] */
    S(10, 11, -M_3J / 2); S(10, 12, M_2J / 2);
    S(11, 10, -M_3J / 2);
    S(12, 10, M_2J / 2);
#undef S
    complete_lt(SM);
}

/* local_mass!, src/FEMMCorotBeamModule.jl:384-554 (the four formulations) */
static void local_mass(double *MM, const double *s, double rho, double L, int mass_type)
{
    const double A = s[0], I1 = s[1], I2 = s[2], I3 = s[3];
    memset(MM, 0, sizeof(double) * 144);
#define U(i, j, v) MM[M12((i) - 1, (j) - 1)] = (v)
#define UA(i, j, v) MM[M12((i) - 1, (j) - 1)] += (v)
    if (mass_type == ORC_BEAM_CONSISTENT_NO_ROT || mass_type == ORC_BEAM_CONSISTENT_WITH_ROT) {
        const double c1 = rho * A * L;
        U(1, 1, c1 * (1.0 / 3)); U(1, 7, c1 * (1.0 / 6));
        U(2, 2, c1 * (13.0 / 35)); U(2, 6, c1 * (11 * L / 210)); U(2, 8, c1 * (9.0 / 70));
        U(2, 12, c1 * (-13 * L / 420));
        U(3, 3, c1 * (13.0 / 35)); U(3, 5, c1 * (-11 * L / 210)); U(3, 9, c1 * (9.0 / 70));
        U(3, 11, c1 * (13 * L / 420));
        U(4, 4, c1 * (I1 / 3 / A)); U(4, 10, c1 * (I1 / 6 / A));
        U(5, 5, c1 * (L * L / 105)); U(5, 9, c1 * (-13 * L / 420)); U(5, 11, c1 * (-L * L / 140));
        U(6, 6, c1 * (L * L / 105)); U(6, 8, c1 * (13 * L / 420)); U(6, 12, c1 * (-L * L / 140));
        U(7, 7, c1 * (1.0 / 3));
        U(8, 8, c1 * (13.0 / 35)); U(8, 12, c1 * (-11 * L / 210));
        U(9, 9, c1 * (13.0 / 35)); U(9, 11, c1 * (11 * L / 210));
        U(10, 10, c1 * (I1 / 3 / A));
        U(11, 11, c1 * (L * L / 105));
        U(12, 12, c1 * (L * L / 105));
        if (mass_type == ORC_BEAM_CONSISTENT_WITH_ROT) {
            const double c2 = rho / L;
            UA(2, 2, c2 * (6.0 / 5 * I2)); UA(2, 6, c2 * (L / 10 * I2)); UA(2, 8, c2 * (-6.0 / 5 * I2));
            UA(2, 12, c2 * (L / 10 * I2));
            UA(3, 3, c2 * (6.0 / 5 * I3)); UA(3, 5, c2 * (-L / 10 * I3)); UA(3, 9, c2 * (-6.0 / 5 * I3));
            UA(3, 11, c2 * (-L / 10 * I3));
            UA(5, 5, c2 * (2 * L * L / 15 * I3)); UA(5, 9, c2 * (L / 10 * I3));
            UA(5, 11, c2 * (-L * L / 30 * I3));
            UA(6, 6, c2 * (2 * L * L / 15 * I2)); UA(6, 8, c2 * (-L / 10 * I2));
            UA(6, 12, c2 * (-L * L / 30 * I2));
            UA(8, 8, c2 * (6.0 / 5 * I2)); UA(8, 12, c2 * (-L / 10 * I2));
            UA(9, 9, c2 * (6.0 / 5 * I3)); UA(9, 11, c2 * (L / 10 * I3));
            UA(11, 11, c2 * (2 * L * L / 15 * I3));
            UA(12, 12, c2 * (2 * L * L / 15 * I2));
        }
        complete_lt(MM);
    } else {
        const double CA = A * rho * L / 2.0;
        const int rot = mass_type == ORC_BEAM_LUMPED_WITH_ROT;
        const double CB = rot ? rho * I1 * L / 2.0 : 0.0;
        const double CC = rot ? rho * I2 * L / 2.0 : 0.0;
        const double CD = rot ? rho * I3 * L / 2.0 : 0.0;
        for (int n = 0; n < 2; n++) {
            UA(6 * n + 1, 6 * n + 1, CA);
            UA(6 * n + 2, 6 * n + 2, CA);
            UA(6 * n + 3, 6 * n + 3, CA);
            if (rot) {
                UA(6 * n + 4, 6 * n + 4, CB);
                UA(6 * n + 5, 6 * n + 5, CC);
                UA(6 * n + 6, 6 * n + 6, CD);
            }
        }
    }
#undef U
#undef UA
}

int orc_beam_element(int which, const double *x0, const double *u, const double *RI,
                     const double *RJ, const double *v, const double *sec, double E, double nu,
                     double rho, int mass_type, double *out)
{
    double xt[6], Ft[9], dN[6];
    for (int k = 0; k < 6; k++) xt[k] = x0[k] + u[k];
    const double G = E / 2 / (1 + nu);
    const double L1 = orc_beam_frame(x0, xt, sec + 7, RI, RJ, Ft, dN);
    const double L0 = sqrt((x0[3] - x0[0]) * (x0[3] - x0[0]) + (x0[4] - x0[1]) * (x0[4] - x0[1]) +
                           (x0[5] - x0[2]) * (x0[5] - x0[2]));
    double aN[72], DN[6], PN[6];
    if (which == ORC_BEAM_STIFFNESS) {
        /* local_stiffness!, :672-677: SM = aN' DN aN */
        cartesian_to_natural(aN, L1);
        natural_stiffness(DN, E, G, sec, L1);
        for (int j = 0; j < 12; j++)
            for (int i = 0; i < 12; i++) {
                double s = 0.0;
                for (int k = 0; k < 6; k++) s += aN[M6(k, i)] * DN[k] * aN[M6(k, j)];
                out[M12(i, j)] = s;
            }
        rotate12(out, Ft);
        return 0;
    }
    if (which == ORC_BEAM_GEOSTIFFNESS || which == ORC_BEAM_RESTORING) {
        /* natural_forces!, :702-707: PN = DN dN */
        natural_stiffness(DN, E, G, sec, L1);
        for (int k = 0; k < 6; k++) PN[k] = DN[k] * dN[k];
        if (which == ORC_BEAM_GEOSTIFFNESS) {
            local_geometric_stiffness(out, PN, L1);
            rotate12(out, Ft);
        } else {
            /* local_forces!, :797-801, then elvec = Te (-LF), :1154 */
            cartesian_to_natural(aN, L1);
            double LF[12];
            for (int i = 0; i < 12; i++) {
                double s = 0.0;
                for (int k = 0; k < 6; k++) s += aN[M6(k, i)] * PN[k];
                LF[i] = -s;
            }
            for (int b = 0; b < 4; b++)
                for (int i = 0; i < 3; i++) {
                    double s = 0.0;
                    for (int k = 0; k < 3; k++) s += Ft[M3(i, k)] * LF[3 * b + k];
                    out[3 * b + i] = s;
                }
        }
        return 0;
    }
    if (which == ORC_BEAM_MASS || which == ORC_BEAM_GYROSCOPIC) {
        double MM[144];
        local_mass(MM, sec, rho, L0, mass_type);
        rotate12(MM, Ft);
        if (which == ORC_BEAM_MASS) {
            memcpy(out, MM, sizeof(MM));
            return 0;
        }
        /* gyroscopic, :883-952: Omega from the nodal velocities in the frame Ft */
        double vf[12]; /* evel1f, 2 x 6 node-major */
        for (int n = 0; n < 2; n++)
            for (int h = 0; h < 2; h++)
                for (int j = 0; j < 3; j++) {
                    double s = 0.0;
                    for (int k = 0; k < 3; k++) s += v[6 * n + 3 * h + k] * Ft[M3(k, j)];
                    vf[6 * n + 3 * h + j] = s;
                }
        double Om[3];
        const double w1 = (vf[3] + vf[6 + 3]) / 2, w2 = (vf[2] - vf[6 + 2]) / L1, w3 = (vf[6 + 1] - vf[1]) / L1;
        for (int c = 0; c < 3; c++) Om[c] = w1 * Ft[M3(c, 0)] + w2 * Ft[M3(c, 1)] + w3 * Ft[M3(c, 2)];
        double OS[9] = {0.0, Om[2], -Om[1], -Om[2], 0.0, Om[0], Om[1], -Om[0], 0.0};
        double OT[144];
        memset(OT, 0, sizeof(OT));
        for (int b = 0; b < 4; b++)
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) OT[M12(3 * b + i, 3 * b + j)] = OS[M3(i, j)];
        for (int j = 0; j < 12; j++)
            for (int i = 0; i < 12; i++) {
                double g1 = 0.0, g2 = 0.0;
                for (int k = 0; k < 12; k++) {
                    g1 += OT[M12(i, k)] * MM[M12(k, j)];
                    g2 += MM[M12(i, k)] * OT[M12(k, j)];
                }
                out[M12(i, j)] = g1 - g2;
            }
        return 0;
    }
    return 1;
}

/* distribloads_global, src/FEMMCorotBeamModule.jl:1186-1247: uniform force
 * per unit length q (global components) -> 12-vector */
int orc_beam_distribload(const double *x0, const double *u, const double *RI, const double *RJ,
                         const double *sec, const double *q, double *out)
{
    double xt[6], Ft[9], dN[6];
    for (int k = 0; k < 6; k++) xt[k] = x0[k] + u[k];
    orc_beam_frame(x0, xt, sec + 7, RI, RJ, Ft, dN);
    const double L0 = sqrt((x0[3] - x0[0]) * (x0[3] - x0[0]) + (x0[4] - x0[1]) * (x0[4] - x0[1]) +
                           (x0[5] - x0[2]) * (x0[5] - x0[2]));
    double Lf[3];
    for (int j = 0; j < 3; j++) Lf[j] = Ft[M3(0, j)] * q[0] + Ft[M3(1, j)] * q[1] + Ft[M3(2, j)] * q[2];
    double f[12] = {Lf[0] * L0 / 2, Lf[1] * L0 / 2, Lf[2] * L0 / 2, 0.0, -Lf[2] * L0 * L0 / 12,
                    +Lf[1] * L0 * L0 / 12, Lf[0] * L0 / 2, Lf[1] * L0 / 2, Lf[2] * L0 / 2, 0.0,
                    +Lf[2] * L0 * L0 / 12, -Lf[1] * L0 * L0 / 12};
    for (int b = 0; b < 4; b++)
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += Ft[M3(i, k)] * f[3 * b + k];
            out[3 * b + i] = s;
        }
    return 0;
}

/* gather element data of element e from the global arrays (Julia layouts) */
static void beam_gather(int64_t e, int64_t nnodes, const double *xyz, const int64_t *conn,
                        const double *u1, const double *R1, const double *v1, double *x0, double *u,
                        double *RI, double *RJ, double *v)
{
    for (int a = 0; a < 2; a++) {
        int64_t node = conn[2 * e + a] - 1;
        for (int c = 0; c < 3; c++) {
            x0[3 * a + c] = xyz[node + c * nnodes];
            u[3 * a + c] = u1 ? u1[node + c * nnodes] : 0.0;
        }
        double *R = a == 0 ? RI : RJ;
        for (int k = 0; k < 9; k++) R[k] = R1 ? R1[node + k * nnodes] : (k % 4 == 0 ? 1.0 : 0.0);
        for (int k = 0; k < 6; k++) v[6 * a + k] = v1 ? v1[node + k * nnodes] : 0.0;
    }
}

int orc_beam_all(int which, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                 const double *u1, const double *R1, const double *v1, const double *sections,
                 double E, double nu, double rho, int mass_type, const double *q, double *out)
{
    int status = 0;
    const int len = (which == ORC_BEAM_RESTORING || which == ORC_BEAM_DISTRIBLOAD) ? 12 : 144;
    for (int64_t e = 0; e < nelem; e++) {
        double x0[6], u[6], RI[9], RJ[9], v[12];
        beam_gather(e, nnodes, xyz, conn, u1, R1, v1, x0, u, RI, RJ, v);
        const double *sec = sections + 10 * e;
        if (which == ORC_BEAM_DISTRIBLOAD)
            status |= orc_beam_distribload(x0, u, RI, RJ, sec, q + 3 * e, out + len * e);
        else
            status |= orc_beam_element(which, x0, u, RI, RJ, v, sec, E, nu, rho, mass_type, out + len * e);
    }
    return status;
}

/* SysvecAssembler: element vectors summed into the global vector in element
 * order; dofs above n are left out */
void orc_assemble_vector(int64_t nnodes, int64_t nelem, int nen, const int64_t *conn,
                         const int64_t *dofnums, int64_t n, const double *Fe, double *F)
{
    memset(F, 0, sizeof(double) * (size_t)(n > 0 ? n : 0));
    for (int64_t e = 0; e < nelem; e++)
        for (int a = 0; a < nen; a++) {
            int64_t node = conn[(int64_t)nen * e + a] - 1;
            for (int k = 0; k < 6; k++) {
                int64_t d = dofnums[node + k * nnodes];
                if (d >= 1 && d <= n) F[d - 1] += Fe[(int64_t)6 * nen * e + 6 * a + k];
            }
        }
}

// Co-rotational beam element math (FEMMCorotBeam), host and device.
//
// The reference (src/FEMMCorotBeamModule.jl) builds every element matrix in
// the element frame Ft and rotates it with the 12x12 block-diagonal
// Te = diag(Ft, Ft, Ft, Ft): K = Te SM Te'.  Here the rotation is applied per
// 3x3 sub-block, K_pq = Ft SM_pq Ft', and the elastic stiffness is written as
// a weighted Gram product: SM = aN' DN aN with a diagonal DN, so
// K = sum_k DN_k g_k g_k' with g_k = Te aN(k,:)' (six 12-vectors).  The
// restoring force is -sum_k PN_k g_k.  Everything is double.
#pragma once

#include <math.h>

#ifndef FS_HD
#if defined(__CUDACC__)
#define FS_HD __host__ __device__ __forceinline__
#else
#define FS_HD inline
#endif
#endif

namespace fs {

// Cross-section of one element (FESetL2Beam fields, src/FESetL2BeamModule.jl:20-31).
struct BeamSection {
    double A, I1, I2, I3, J, A2s, A3s;
    double x1x2[3];
};

struct BeamFrame {
    double Ft[3][3];  // current element frame, columns = axes
    double L0, L1;    // initial and current length
    double dN[6];     // natural deformations
};

FS_HD double bm_norm3(const double v[3])
{
    return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

// axis 3 = axis 1 x v normalised, axis 2 = axis 3 x axis 1 (the explicit
// skew products of src/FESetL2BeamModule.jl:112-125, src/FEMMCorotBeamModule.jl:161-180)
FS_HD void bm_complete_frame(double F[3][3], const double v[3])
{
    double e3[3] = {F[1][0] * v[2] - F[2][0] * v[1], F[2][0] * v[0] - F[0][0] * v[2],
                    F[0][0] * v[1] - F[1][0] * v[0]};
    const double n3 = bm_norm3(e3);
    for (int i = 0; i < 3; i++) F[i][2] = e3[i] / n3;
    F[0][1] = F[1][2] * F[2][0] - F[2][2] * F[1][0];
    F[1][1] = F[2][2] * F[0][0] - F[0][2] * F[2][0];
    F[2][1] = F[0][2] * F[1][0] - F[1][2] * F[0][0];
}

// local_frame_and_def! (src/FEMMCorotBeamModule.jl:208-243): current frame,
// lengths and natural deformations from the initial and current nodal
// positions and the nodal rotation matrices RI, RJ.
FS_HD void beam_frame(const double x0[2][3], const double xt[2][3], const double x1x2[3],
                                           const double RI[3][3], const double RJ[3][3], BeamFrame &f)
{
    double F0[3][3], d[3];
    for (int c = 0; c < 3; c++) d[c] = x0[1][c] - x0[0][c];
    f.L0 = bm_norm3(d);
    for (int c = 0; c < 3; c++) F0[c][0] = d[c] / f.L0;
    bm_complete_frame(F0, x1x2);
    // nodal cross-section frames FtI = RI F0, FtJ = RJ F0
    double FI[3][3], FJ[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double si = 0.0, sj = 0.0;
            for (int k = 0; k < 3; k++) {
                si += RI[i][k] * F0[k][j];
                sj += RJ[i][k] * F0[k][j];
            }
            FI[i][j] = si;
            FJ[i][j] = sj;
        }
    for (int c = 0; c < 3; c++) d[c] = xt[1][c] - xt[0][c];
    f.L1 = bm_norm3(d);
    for (int c = 0; c < 3; c++) f.Ft[c][0] = d[c] / f.L1;
    double v[3] = {FI[0][1] + FJ[0][1], FI[1][1] + FJ[1][1], FI[2][1] + FJ[2][1]};
    bm_complete_frame(f.Ft, v);
    // components of the nodal frames in the element frame: L = Ft' F
    double LI[3][3], LJ[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double si = 0.0, sj = 0.0;
            for (int k = 0; k < 3; k++) {
                si += f.Ft[k][i] * FI[k][j];
                sj += f.Ft[k][i] * FJ[k][j];
            }
            LI[i][j] = si;
            LJ[i][j] = sj;
        }
    f.dN[0] = f.L1 - f.L0;
    f.dN[5] = (LJ[2][1] / LJ[1][1] - LI[2][1] / LI[1][1] - LJ[1][2] / LJ[2][2] + LI[1][2] / LI[2][2]) / 2;
    const double TH2I = -LI[2][0] / LI[0][0], TH2J = -LJ[2][0] / LJ[0][0];
    const double TH3I = LI[1][0] / LI[0][0], TH3J = LJ[1][0] / LJ[0][0];
    f.dN[1] = TH3I - TH3J;
    f.dN[2] = TH3I + TH3J;
    f.dN[3] = -TH2I + TH2J;
    f.dN[4] = -TH2I - TH2J;
}

// natural_stiffness! (src/FEMMCorotBeamModule.jl:729-779): diagonal DN,
// Bernoulli when either shear area is infinite, else Timoshenko.
FS_HD void beam_natural_stiffness(const BeamSection &s, double E, double G, double L,
                                                                double DN[6])
{
    DN[0] = E * s.A / L;
    DN[1] = E * s.I3 / L;
    DN[3] = E * s.I2 / L;
    DN[5] = G * s.J / L;
    if (isinf(s.A2s) || isinf(s.A3s)) {
        DN[2] = 3 * E * s.I3 / L;
        DN[4] = 3 * E * s.I2 / L;
    } else {
        const double Phi3 = 12 * E * s.I3 / (G * s.A2s * L * L);
        const double Phi2 = 12 * E * s.I2 / (G * s.A3s * L * L);
        DN[2] = 3 * E * s.I3 / L / (1 + Phi3);
        DN[4] = 3 * E * s.I2 / L / (1 + Phi2);
    }
}

// Row k of local_cartesian_to_natural! (src/FEMMCorotBeamModule.jl:265-289)
// rotated to global components: g[12] = Te aN(k,:)'.  Each row of aN has at
// most two nonzero 3-vectors; g's sub-vector p is Ft times aN's.
FS_HD void beam_row(int k, const double Ft[3][3], double L, double g[12])
{
    // local sub-vectors of row k (4 sub-vectors of 3)
    double a[12];
    for (int i = 0; i < 12; i++) a[i] = 0.0;
    switch (k) {
    case 0: a[0] = -1; a[6] = 1; break;
    case 1: a[5] = 1; a[11] = -1; break;
    case 2: a[1] = 2 / L; a[5] = 1; a[7] = -2 / L; a[11] = 1; break;
    case 3: a[4] = -1; a[10] = 1; break;
    case 4: a[2] = 2 / L; a[4] = -1; a[8] = -2 / L; a[10] = -1; break;
    default: a[3] = -1; a[9] = 1; break;
    }
    for (int p = 0; p < 4; p++)
        for (int i = 0; i < 3; i++)
            g[3 * p + i] = Ft[i][0] * a[3 * p] + Ft[i][1] * a[3 * p + 1] + Ft[i][2] * a[3 * p + 2];
}

// Entry (i, j) (0-based, any order) of local_geometric_stiffness!
// (src/FEMMCorotBeamModule.jl:321-382) for the natural forces PN.
FS_HD double beam_geo_entry(int i, int j, const double PN[6], double L)
{
    if (i > j) {
        int t = i;
        i = j;
        j = t;
    }
    const double N = PN[0], S_2 = -2 * PN[2] / L, S_3 = -2 * PN[4] / L, M_1 = PN[5];
    const double M_2I = PN[3] + PN[4], M_2J = PN[3] - PN[4];
    const double M_3I = -(PN[1] + PN[2]), M_3J = -(PN[1] - PN[2]);
    switch (i * 12 + j) {
    // [1:3, 1:3] and [7:9, 7:9]
    case 0 * 12 + 1: case 6 * 12 + 7: return -S_2 / L;
    case 0 * 12 + 2: case 6 * 12 + 8: return -S_3 / L;
    case 1 * 12 + 1: case 2 * 12 + 2: case 7 * 12 + 7: case 8 * 12 + 8: return N / L;
    // [1:3, 4:6]
    case 1 * 12 + 3: return -M_2I / L;
    case 1 * 12 + 4: return M_1 / L;
    case 2 * 12 + 3: return -M_3I / L;
    case 2 * 12 + 5: return M_1 / L;
    // [1:3, 7:9]
    case 0 * 12 + 7: case 1 * 12 + 6: return S_2 / L;
    case 0 * 12 + 8: case 2 * 12 + 6: return S_3 / L;
    case 1 * 12 + 7: case 2 * 12 + 8: return -N / L;
    // [1:3, 10:12]
    case 1 * 12 + 9: return M_2J / L;
    case 1 * 12 + 10: return -M_1 / L;
    case 2 * 12 + 9: return M_3J / L;
    case 2 * 12 + 11: return -M_1 / L;
    // [4:6, 4:6]
    case 3 * 12 + 4: return M_3I / 2;
    case 3 * 12 + 5: return -M_2I / 2;
    // [4:6, 7:9]
    case 3 * 12 + 7: return M_2I / L;
    case 3 * 12 + 8: return M_3I / L;
    case 4 * 12 + 7: return -M_1 / L;
    case 5 * 12 + 8: return -M_1 / L;
    // [4:6, 10:12]
    case 4 * 12 + 11: return M_1 / 2;
    case 5 * 12 + 10: return -M_1 / 2;
    // [7:9, 10:12]
    case 7 * 12 + 9: return -M_2J / L;
    case 7 * 12 + 10: return M_1 / L;
    case 8 * 12 + 9: return -M_3J / L;
    case 8 * 12 + 11: return M_1 / L;
    // [10:12, 10:12]
    case 9 * 12 + 10: return -M_3J / 2;
    case 9 * 12 + 11: return M_2J / 2;
    default: return 0.0;
    }
}

// Entry (i, j) of local_mass! (src/FEMMCorotBeamModule.jl:384-554) for the
// four formulations (mass_type 0..3 of :144-147); L is the initial length.
FS_HD double beam_mass_entry(int i, int j, const BeamSection &s, double rho, double L,
                                                  int mass_type)
{
    if (i > j) {
        int t = i;
        i = j;
        j = t;
    }
    if (mass_type >= 2) {  // lumped diagonal
        if (i != j) return 0.0;
        const int k = i % 6;
        if (k < 3) return s.A * rho * L / 2.0;
        if (mass_type == 2) return 0.0;
        const double I = k == 3 ? s.I1 : (k == 4 ? s.I2 : s.I3);
        return rho * I * L / 2.0;
    }
    const double c1 = rho * s.A * L;
    double v = 0.0;
    switch (i * 12 + j) {
    case 0 * 12 + 0: case 6 * 12 + 6: v = c1 * (1.0 / 3); break;
    case 0 * 12 + 6: v = c1 * (1.0 / 6); break;
    case 1 * 12 + 1: case 2 * 12 + 2: case 7 * 12 + 7: case 8 * 12 + 8: v = c1 * (13.0 / 35); break;
    case 1 * 12 + 5: case 8 * 12 + 10: v = c1 * (11 * L / 210); break;
    case 2 * 12 + 4: case 7 * 12 + 11: v = c1 * (-11 * L / 210); break;
    case 1 * 12 + 7: case 2 * 12 + 8: v = c1 * (9.0 / 70); break;
    case 1 * 12 + 11: case 4 * 12 + 8: v = c1 * (-13 * L / 420); break;
    case 2 * 12 + 10: case 5 * 12 + 7: v = c1 * (13 * L / 420); break;
    case 3 * 12 + 3: case 9 * 12 + 9: v = c1 * (s.I1 / 3 / s.A); break;
    case 3 * 12 + 9: v = c1 * (s.I1 / 6 / s.A); break;
    case 4 * 12 + 4: case 5 * 12 + 5: case 10 * 12 + 10: case 11 * 12 + 11: v = c1 * (L * L / 105); break;
    case 4 * 12 + 10: case 5 * 12 + 11: v = c1 * (-L * L / 140); break;
    default: break;
    }
    if (mass_type == 1) {  // rotary inertia of the cross-section
        const double c2 = rho / L;
        switch (i * 12 + j) {
        case 1 * 12 + 1: case 7 * 12 + 7: v += c2 * (6.0 / 5 * s.I2); break;
        case 1 * 12 + 5: case 1 * 12 + 11: v += c2 * (L / 10 * s.I2); break;
        case 1 * 12 + 7: v += c2 * (-6.0 / 5 * s.I2); break;
        case 2 * 12 + 2: case 8 * 12 + 8: v += c2 * (6.0 / 5 * s.I3); break;
        case 2 * 12 + 4: case 2 * 12 + 10: v += c2 * (-L / 10 * s.I3); break;
        case 2 * 12 + 8: v += c2 * (-6.0 / 5 * s.I3); break;
        case 4 * 12 + 4: case 10 * 12 + 10: v += c2 * (2 * L * L / 15 * s.I3); break;
        case 4 * 12 + 8: case 8 * 12 + 10: v += c2 * (L / 10 * s.I3); break;
        case 4 * 12 + 10: v += c2 * (-L * L / 30 * s.I3); break;
        case 5 * 12 + 5: case 11 * 12 + 11: v += c2 * (2 * L * L / 15 * s.I2); break;
        case 5 * 12 + 7: case 7 * 12 + 11: v += c2 * (-L / 10 * s.I2); break;
        case 5 * 12 + 11: v += c2 * (-L * L / 30 * s.I2); break;
        default: break;
        }
    }
    return v;
}

// out = Ft S Ft' for a 3x3 S
FS_HD void bm_rotate3(const double Ft[3][3], const double S[3][3], double out[3][3])
{
    double T[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T[i][j] = S[i][0] * Ft[j][0] + S[i][1] * Ft[j][1] + S[i][2] * Ft[j][2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[i][j] = Ft[i][0] * T[0][j] + Ft[i][1] * T[1][j] + Ft[i][2] * T[2][j];
}

// Everything one element needs to produce its node blocks.
struct BeamElem {
    BeamFrame f;
    BeamSection s;
    double DN[6];     // natural stiffness (at the current length)
    double PN[6];     // natural forces DN dN
    double OS[3][3];  // skew matrix of the frame's angular velocity (gyroscopic)
    double rho;
    int mass_type;
};

// x0, xt: initial and current nodal positions; R: nodal rotation matrices;
// v: nodal velocities (6 per node, gyroscopic only; null for none).
FS_HD void beam_prepare(const double x0[2][3], const double xt[2][3], const double R[2][3][3], const double (*v)[6],
                        const BeamSection &s, double E, double G, double rho, int mass_type, BeamElem &e)
{
    e.s = s;
    e.rho = rho;
    e.mass_type = mass_type;
    beam_frame(x0, xt, s.x1x2, R[0], R[1], e.f);
    beam_natural_stiffness(s, E, G, e.f.L1, e.DN);
    for (int k = 0; k < 6; k++) e.PN[k] = e.DN[k] * e.f.dN[k];
    // angular velocity of the element frame from the nodal velocities
    // (gyroscopic, src/FEMMCorotBeamModule.jl:926-935)
    double vf[2][6];
    for (int a = 0; a < 2; a++)
        for (int h = 0; h < 2; h++)
            for (int j = 0; j < 3; j++)
                vf[a][3 * h + j] = v ? v[a][3 * h] * e.f.Ft[0][j] + v[a][3 * h + 1] * e.f.Ft[1][j] +
                                           v[a][3 * h + 2] * e.f.Ft[2][j]
                                     : 0.0;
    const double w1 = (vf[0][3] + vf[1][3]) / 2, w2 = (vf[0][2] - vf[1][2]) / e.f.L1,
                 w3 = (vf[1][1] - vf[0][1]) / e.f.L1;
    double Om[3];
    for (int c = 0; c < 3; c++) Om[c] = w1 * e.f.Ft[c][0] + w2 * e.f.Ft[c][1] + w3 * e.f.Ft[c][2];
    e.OS[0][0] = 0.0;    e.OS[0][1] = -Om[2]; e.OS[0][2] = Om[1];
    e.OS[1][0] = Om[2];  e.OS[1][1] = 0.0;    e.OS[1][2] = -Om[0];
    e.OS[2][0] = -Om[1]; e.OS[2][1] = Om[0];  e.OS[2][2] = 0.0;
}

// Node block (a, b) of the global element matrix WHICH (0 stiffness,
// 1 geometric stiffness, 2 mass, 3 gyroscopic): acc[i][j] = K[6a+i][6b+j].
template <int WHICH>
FS_HD void beam_block_raw(const BeamElem &e, int a, int b, double acc[6][6])
{
    if (WHICH == 0) {
        // K = sum_k DN_k g_k g_k'
        double g[6][12];
        for (int k = 0; k < 6; k++) beam_row(k, e.f.Ft, e.f.L1, g[k]);
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++) {
                double v = 0.0;
                for (int k = 0; k < 6; k++) v += e.DN[k] * g[k][6 * a + i] * g[k][6 * b + j];
                acc[i][j] = v;
            }
        return;
    }
    for (int pp = 0; pp < 2; pp++)
        for (int qq = 0; qq < 2; qq++) {
            double S[3][3], K[3][3];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    const int gi = 6 * a + 3 * pp + i, gj = 6 * b + 3 * qq + j;
                    S[i][j] = WHICH == 1 ? beam_geo_entry(gi, gj, e.PN, e.f.L1)
                                         : beam_mass_entry(gi, gj, e.s, e.rho, e.f.L0, e.mass_type);
                }
            bm_rotate3(e.f.Ft, S, K);
            if (WHICH == 3) {
                // Ge_pq = OS M_pq - M_pq OS
                double G3[3][3];
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        double g1 = 0.0, g2 = 0.0;
                        for (int k = 0; k < 3; k++) {
                            g1 += e.OS[i][k] * K[k][j];
                            g2 += K[i][k] * e.OS[k][j];
                        }
                        G3[i][j] = g1 - g2;
                    }
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) K[i][j] = G3[i][j];
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) acc[3 * pp + i][3 * qq + j] = K[i][j];
        }
}

// Node block (a, b); a diagonal block is made exactly symmetric from its
// upper triangle (as complete_lt! does), so the assembled matrix is symmetric
// to the bit.
template <int WHICH>
FS_HD void beam_block(const BeamElem &e, int a, int b, double acc[6][6])
{
    beam_block_raw<WHICH>(e, a, b, acc);
    if (a == b)
        for (int i = 0; i < 6; i++)
            for (int j = i + 1; j < 6; j++) acc[j][i] = acc[i][j];
}

// Restoring force -Te aN' PN (restoringforce, src/FEMMCorotBeamModule.jl:1112-1159).
FS_HD void beam_restoring(const BeamElem &e, double out[12])
{
    for (int i = 0; i < 12; i++) out[i] = 0.0;
    for (int k = 0; k < 6; k++) {
        double g[12];
        beam_row(k, e.f.Ft, e.f.L1, g);
        for (int i = 0; i < 12; i++) out[i] -= e.PN[k] * g[i];
    }
}

// Consistent nodal loads of a uniform force per unit length q (global
// components): distribloads_global (src/FEMMCorotBeamModule.jl:1186-1247).
FS_HD void beam_distribload(const BeamElem &e, const double q[3], double out[12])
{
    const double(&Ft)[3][3] = e.f.Ft;
    double Lf[3];
    for (int j = 0; j < 3; j++) Lf[j] = Ft[0][j] * q[0] + Ft[1][j] * q[1] + Ft[2][j] * q[2];
    const double L0 = e.f.L0;
    const double fl[12] = {Lf[0] * L0 / 2, Lf[1] * L0 / 2, Lf[2] * L0 / 2, 0.0, -Lf[2] * L0 * L0 / 12,
                           +Lf[1] * L0 * L0 / 12, Lf[0] * L0 / 2, Lf[1] * L0 / 2, Lf[2] * L0 / 2, 0.0,
                           +Lf[2] * L0 * L0 / 12, -Lf[1] * L0 * L0 / 12};
    for (int p = 0; p < 4; p++)
        for (int i = 0; i < 3; i++)
            out[3 * p + i] = Ft[i][0] * fl[3 * p] + Ft[i][1] * fl[3 * p + 1] + Ft[i][2] * fl[3 * p + 2];
}

}  // namespace fs

// Test-only host build of the CUDA library's per-element math
// (csrc/fs_elem_math.cuh), so the restructured Gram-row formulation can be
// compared with the oracle on a machine without a GPU.  Not part of the
// product: the library itself has no CPU path.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "fs_host_prep.h"
#include "fs_beam_math.cuh"
#include "fs_comp_sum.cuh"

using namespace fs;

// How the Gram K = sum_r row_r row_r^T of an element is summed.
enum GramSum {
    GRAM_PLAIN,  // in the row type, rows in order (FS_FP64, FS_MIXED)
    GRAM_COMP,   // FS_MIXED_COMP: the kernels' compensated sums (fs_comp_sum.cuh)
    GRAM_EXACT,  // float rows: products exact in double, summed in double
    GRAM_ABS     // float rows: sum of |row_r[i] row_r[j]| (error bounds)
};

// The element kernels' FS_MIXED_COMP sums: entries (i, 2q) and (i, 2q + 1)
// packed in one f32x2 and summed over the rows in order at LEVELS levels,
// the pairs holding an entry j >= i only, then the upper triangle mirrored;
// each entry the double nearest hi + lo (one rounding).
template <int LEVELS>
static void comp_gram(const float (*rows)[24], int nrows, int nd, double *K)
{
    for (int i = 0; i < nd; i++)
        for (int q = 0; 2 * q < nd; q++) {
            if (2 * q + 1 < i) continue;
            f32x2 s = x2_pack(0.f, 0.f), c = s, d = s, hh, ll;
            for (int r = 0; r < nrows; r++) {
                const f32x2 a2 = x2_pack(rows[r][i], rows[r][i]), na2 = x2_pack(-rows[r][i], -rows[r][i]);
                const f32x2 b2 = x2_pack(rows[r][2 * q], rows[r][2 * q + 1]);
                if (LEVELS == 3)
                    dot3_step_x2(s, c, d, a2, na2, b2);
                else
                    dot2_step_x2(s, c, a2, na2, b2);
            }
            x2_pair_finish<LEVELS>(s, c, d, hh, ll);
            float h0, h1, l0, l1;
            x2_unpack(hh, h0, h1);
            x2_unpack(ll, l0, l1);
            K[i + nd * (2 * q)] = (double)h0 + (double)l0;
            K[i + nd * (2 * q + 1)] = (double)h1 + (double)l1;
        }
    for (int j = 0; j < nd; j++)
        for (int i = j + 1; i < nd; i++) K[i + nd * j] = K[j + nd * i];
}

template <class R, bool FFRAME = false>
static int elem_matrices(int etype, int64_t nnodes, const double *xyz, int64_t nelem,
                         const int64_t *conn, const double *normals, const uint8_t *valid,
                         const double *thick, const fs_shell_params *p, const fs_layup_group *groups,
                         const int32_t *egroup, double *out, GramSum gram = GRAM_PLAIN)
{
    MatConst mc;
    if (prepare_matconst(*p, mc)) return 1;
    bool comp = (etype == FS_T3FFCOMP || etype == FS_Q4RSCOMP);
    int ng = 0;
    if (comp)
        for (int64_t e = 0; e < nelem; e++) ng = egroup[e] + 1 > ng ? egroup[e] + 1 : ng;
    std::vector<GroupConst> gcs(ng > 0 ? ng : 1);
    for (int g = 0; g < ng; g++)
        if (prepare_group(groups[g], gcs[g])) return 1;
    int nn = (etype == FS_T3FF || etype == FS_T3FFCOMP) ? 3 : 4;
    int nd = 6 * nn;
    for (int64_t e = 0; e < nelem; e++) {
        const GroupConst *gc = comp ? &gcs[egroup[e]] : nullptr;
        const int nrows_max = 40;
        R rows[nrows_max][24];
        memset(rows, 0, sizeof(rows));
        int nrows = 0, st = 0;
        if (nn == 3) {
            ElemIn<3> in;
            for (int a = 0; a < 3; a++) {
                int64_t node = conn[3 * e + a] - 1;
                for (int c = 0; c < 3; c++) {
                    in.X[a][c] = xyz[node + c * nnodes];
                    in.nrm[a][c] = normals[node + c * nnodes];
                    in.nrmf[a][c] = (float)in.nrm[a][c];
                }
                in.valid[a] = valid[node] != 0;
            }
            in.t = thick[e];
            if (p->transv_shear_formulation == 1) {
                nrows = T3Rows<true>::N;
                st = comp ? t3_rows<R, true, true>(in, mc, gc, &rows[0][0], 24)
                          : t3_rows<R, false, true>(in, mc, gc, &rows[0][0], 24);
            } else {
                nrows = T3Rows<false>::N;
                st = comp ? t3_rows<R, true, false>(in, mc, gc, &rows[0][0], 24)
                          : t3_rows<R, false, false>(in, mc, gc, &rows[0][0], 24);
            }
        } else {
            ElemIn<4> in;
            for (int a = 0; a < 4; a++) {
                int64_t node = conn[4 * e + a] - 1;
                for (int c = 0; c < 3; c++) {
                    in.X[a][c] = xyz[node + c * nnodes];
                    in.nrm[a][c] = normals[node + c * nnodes];
                    in.nrmf[a][c] = (float)in.nrm[a][c];
                }
                in.valid[a] = valid[node] != 0;
            }
            in.t = thick[e];
            Q4Elem qe;
            q4_prepare(in, comp ? gc->thickness : in.t, mc.stab_c, qe);
            double tr[4] = {0, 0, 0, 0};
            float trf[4] = {0, 0, 0, 0};
            for (int j = 0; j < 4; j++) {
                double trj[4];
                st |= comp ? q4_point_rows<R, true, false, FFRAME>(in, qe, j, mc, gc, &rows[8 * j][0], 24, trj)
                           : q4_point_rows<R, false, false, FFRAME>(in, qe, j, mc, gc, &rows[8 * j][0], 24, trj);
                for (int k = 0; k < 4; k++) {
                    tr[k] += trj[k];
                    trf[k] += (float)trj[k];
                }
            }
            if constexpr (FFRAME)
                q4_drill_rows_f(in, trf, (float)mc.drill_scale, &rows[32][0], 24);
            else
                q4_drill_rows<R>(in, tr, mc.drill_scale, &rows[32][0], 24);
            nrows = 36;
        }
        if (st) return 10 + st;
        double *K = out + (int64_t)nd * nd * e;
        if constexpr (sizeof(R) == 4) {
            if (gram == GRAM_COMP) {
                if (nn == 3)
                    comp_gram<T3_PAIR_LEVELS>(rows, nrows, nd, K);
                else
                    comp_gram<Q4_PAIR_LEVELS>(rows, nrows, nd, K);
                continue;
            }
        }
        for (int j = 0; j < nd; j++)
            for (int i = 0; i < nd; i++) {
                if (gram == GRAM_EXACT || gram == GRAM_ABS) {
                    // products of float rows are exact in double; summed in
                    // long double (a significand of 64 bits or more: at most
                    // 36 terms, within 2^-58 of their magnitudes), rounded
                    // once to double
                    long double s = 0;
                    for (int r = 0; r < nrows; r++) {
                        const double t = (double)rows[r][i] * (double)rows[r][j];
                        s += gram == GRAM_ABS ? fabs(t) : t;
                    }
                    K[i + nd * j] = (double)s;
                } else {
                    R s = 0;
                    for (int r = 0; r < nrows; r++) s += rows[r][i] * rows[r][j];
                    K[i + nd * j] = (double)s;
                }
            }
    }
    return 0;
}

extern "C" int hc_element_matrices(int etype, int precision, int64_t nnodes, const double *xyz,
                                   int64_t nelem, const int64_t *conn, const double *normals,
                                   const uint8_t *valid, const double *thick,
                                   const fs_shell_params *p, const fs_layup_group *groups,
                                   const int32_t *egroup, double *out)
{
    if (precision == FS_FP64)
        return elem_matrices<double>(etype, nnodes, xyz, nelem, conn, normals, valid, thick, p, groups,
                                     egroup, out);
    // FS_MIXED: the Q4 points' frames in float, as the library's FS_MIXED
    // kernel; FS_MIXED_COMP: double frames, float rows, the kernels'
    // compensated sums.  Test-only precisions 3 and 4: the FS_MIXED_COMP rows'
    // exact Gram, and the sums of |row_r[i] row_r[j]| of those rows.
    if (precision == FS_MIXED)
        return elem_matrices<float, true>(etype, nnodes, xyz, nelem, conn, normals, valid, thick, p, groups,
                                          egroup, out);
    const GramSum g = precision == FS_MIXED_COMP ? GRAM_COMP : precision == 3 ? GRAM_EXACT : GRAM_ABS;
    if (precision != FS_MIXED_COMP && precision != 3 && precision != 4) return 2;
    return elem_matrices<float>(etype, nnodes, xyz, nelem, conn, normals, valid, thick, p, groups,
                                egroup, out, g);
}

// The compensated dot product of the element kernels on both lanes of an
// f32x2: (a . b0, a . b1) summed in order at `levels` levels (2: Dot2, 3),
// out = {hi0, lo0, hi1, lo1}.
extern "C" int hc_comp_dot(int levels, int n, const float *a, const float *b0, const float *b1, float *out)
{
    if (levels != 2 && levels != 3) return 1;
    f32x2 s = x2_pack(0.f, 0.f), c = s, d = s, hh, ll;
    for (int r = 0; r < n; r++) {
        const f32x2 a2 = x2_pack(a[r], a[r]), na2 = x2_pack(-a[r], -a[r]), b2 = x2_pack(b0[r], b1[r]);
        if (levels == 3)
            dot3_step_x2(s, c, d, a2, na2, b2);
        else
            dot2_step_x2(s, c, a2, na2, b2);
    }
    if (levels == 3)
        x2_pair_finish<3>(s, c, d, hh, ll);
    else
        x2_pair_finish<2>(s, c, d, hh, ll);
    x2_unpack(hh, out[0], out[2]);
    x2_unpack(ll, out[1], out[3]);
    return 0;
}

// The gather's column sum of float-pair entries on both lanes of an f32x2:
// lane k sums the pairs (hi[k n + r], lo[k n + r]), r < n, as a float triple
// (the first pair taken as is, the next ones by x2_triple_add) and rounds it
// to double: out[k].
extern "C" int hc_triple_sum(int n, const float *hi, const float *lo, double *out)
{
    if (n < 1) return 1;
    f32x2 h = x2_pack(hi[0], hi[n]), l = x2_pack(lo[0], lo[n]), t = x2_pack(0.f, 0.f);
    for (int r = 1; r < n; r++) x2_triple_add(h, l, t, x2_pack(hi[r], hi[n + r]), x2_pack(lo[r], lo[n + r]));
    float h0, h1, l0, l1, t0, t1;
    x2_unpack(h, h0, h1);
    x2_unpack(l, l0, l1);
    x2_unpack(t, t0, t1);
    out[0] = triple_value(h0, l0, t0);
    out[1] = triple_value(h1, l1, t1);
    return 0;
}

// Stress resultants at the integration points (the device point math of
// csrc/fs_elem_math.cuh): quantity 1 moment, 2 shear, 3 membrane; u nnodes x 6
// column-major; cs one 3x3 column-major matrix (ncs = 1), one per point, or
// none (ncs = 0: the element frame at the point).
extern "C" int hc_resultants(int etype, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                             const double *normals, const uint8_t *valid, const double *thick,
                             const fs_shell_params *p, const double *u, int quant, const double *cs, int64_t ncs,
                             double *out)
{
    MatConst mc;
    if (prepare_matconst(*p, mc)) return 1;
    const int nn = etype == FS_T3FF ? 3 : 4, npt = nn == 3 ? 1 : 4;
    for (int64_t e = 0; e < nelem; e++) {
        double ue[24];
        for (int a = 0; a < nn; a++)
            for (int k = 0; k < 6; k++) ue[6 * a + k] = u[(conn[nn * e + a] - 1) + k * nnodes];
        if (nn == 3) {
            ElemIn<3> in;
            for (int a = 0; a < 3; a++) {
                int64_t node = conn[3 * e + a] - 1;
                for (int c = 0; c < 3; c++) {
                    in.X[a][c] = xyz[node + c * nnodes];
                    in.nrm[a][c] = normals[node + c * nnodes];
                    in.nrmf[a][c] = (float)in.nrm[a][c];
                }
                in.valid[a] = valid[node] != 0;
            }
            in.t = thick[e];
            t3_resultant(in, mc, ue, quant, ncs == 0 ? nullptr : (ncs == 1 ? cs : cs + 9 * e), out + 3 * e);
        } else {
            ElemIn<4> in;
            for (int a = 0; a < 4; a++) {
                int64_t node = conn[4 * e + a] - 1;
                for (int c = 0; c < 3; c++) {
                    in.X[a][c] = xyz[node + c * nnodes];
                    in.nrm[a][c] = normals[node + c * nnodes];
                    in.nrmf[a][c] = (float)in.nrm[a][c];
                }
                in.valid[a] = valid[node] != 0;
            }
            in.t = thick[e];
            Q4Elem qe;
            q4_prepare(in, in.t, mc.stab_c, qe);
            for (int j = 0; j < 4; j++) {
                const int64_t q = npt * e + j;
                if (q4_resultant(in, qe, j, mc, ue, quant, ncs == 0 ? nullptr : (ncs == 1 ? cs : cs + 9 * q), out + 3 * q))
                    return 4;
            }
        }
    }
    return 0;
}

extern "C" int hc_lumped(int etype, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                         const double *thick, double rho, const fs_layup_group *groups,
                         const int32_t *egroup, double *out)
{
    bool comp = (etype == FS_T3FFCOMP || etype == FS_Q4RSCOMP);
    int nn = (etype == FS_T3FF || etype == FS_T3FFCOMP) ? 3 : 4;
    for (int64_t e = 0; e < nelem; e++) {
        GroupConst gc;
        if (comp) prepare_group(groups[egroup[e]], gc);
        if (nn == 3) {
            ElemIn<3> in;
            for (int a = 0; a < 3; a++)
                for (int c = 0; c < 3; c++) in.X[a][c] = xyz[(conn[3 * e + a] - 1) + c * nnodes];
            in.t = thick[e];
            lumped_mass<3>(in, rho, comp, &gc, out[2 * e], out[2 * e + 1]);
        } else {
            ElemIn<4> in;
            for (int a = 0; a < 4; a++)
                for (int c = 0; c < 3; c++) in.X[a][c] = xyz[(conn[4 * e + a] - 1) + c * nnodes];
            in.t = thick[e];
            lumped_mass<4>(in, rho, comp, &gc, out[2 * e], out[2 * e + 1]);
        }
    }
    return 0;
}

// Beam element matrices (which 0..3, 12x12 column-major each) or vectors
// (which 4 restoring force, 5 distributed load q[3] per element) from the
// library's beam math (csrc/fs_beam_math.cuh).  Layouts as the oracle's.
extern "C" int hc_beam_elements(int which, int64_t nnodes, const double *xyz, int64_t nelem,
                                const int64_t *conn, const double *u1, const double *R1,
                                const double *v1, const double *sections, double E, double nu,
                                double rho, int mass_type, const double *q, double *out)
{
    const double G = E / 2 / (1 + nu);
    for (int64_t e = 0; e < nelem; e++) {
        double x0[2][3], xt[2][3], R[2][3][3], v[2][6];
        for (int a = 0; a < 2; a++) {
            int64_t node = conn[2 * e + a] - 1;
            for (int c = 0; c < 3; c++) {
                x0[a][c] = xyz[node + c * nnodes];
                xt[a][c] = x0[a][c] + (u1 ? u1[node + c * nnodes] : 0.0);
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    R[a][i][j] = R1 ? R1[node + (i + 3 * j) * nnodes] : (i == j ? 1.0 : 0.0);
            for (int k = 0; k < 6; k++) v[a][k] = v1 ? v1[node + k * nnodes] : 0.0;
        }
        BeamSection s;
        memcpy(&s, sections + 10 * e, sizeof(s));
        BeamElem el;
        beam_prepare(x0, xt, R, v, s, E, G, rho, mass_type, el);
        if (which >= 4) {
            if (which == 4)
                beam_restoring(el, out + 12 * e);
            else
                beam_distribload(el, q + 3 * e, out + 12 * e);
            continue;
        }
        double *K = out + 144 * e;
        for (int a = 0; a < 2; a++)
            for (int b = a; b < 2; b++) {
                double acc[6][6];
                switch (which) {
                case 0: beam_block<0>(el, a, b, acc); break;
                case 1: beam_block<1>(el, a, b, acc); break;
                case 2: beam_block<2>(el, a, b, acc); break;
                default: beam_block<3>(el, a, b, acc); break;
                }
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++) {
                        K[(6 * a + i) + 12 * (6 * b + j)] = acc[i][j];
                        K[(6 * b + j) + 12 * (6 * a + i)] = acc[i][j];
                    }
            }
    }
    return 0;
}

// Q4 basis gradients at the four Gauss points: tabulated (out[0..31]) and
// computed (out[32..63]), gp[j][a][k]
extern "C" void hc_q4_basis(double *out)
{
    for (int j = 0; j < 4; j++) {
        double xi, eta, a[4][2], b[4][2];
        q4_point(j, xi, eta);
        q4_dbasis_gp(j, a);
        q4_dbasis(xi, eta, b);
        for (int n = 0; n < 4; n++)
            for (int k = 0; k < 2; k++) {
                out[8 * j + 2 * n + k] = a[n][k];
                out[32 + 8 * j + 2 * n + k] = b[n][k];
            }
    }
}

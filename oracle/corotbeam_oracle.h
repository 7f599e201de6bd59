/*
 * CPU oracle for the co-rotational beam element loops (FEMMCorotBeam).
 * TEST INFRASTRUCTURE ONLY; see corotbeam_oracle.c.
 *
 * A cross section is 10 doubles per element: A, I1, I2, I3, J, A2s, A3s and
 * the x1x2_vector (FESetL2Beam fields, src/FESetL2BeamModule.jl:20-31).
 */
#ifndef COROTBEAM_ORACLE_H
#define COROTBEAM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_BEAM_STIFFNESS = 0,
    ORC_BEAM_GEOSTIFFNESS = 1,
    ORC_BEAM_MASS = 2,
    ORC_BEAM_GYROSCOPIC = 3,
    ORC_BEAM_RESTORING = 4,
    ORC_BEAM_DISTRIBLOAD = 5
};

/* mass formulations, src/FEMMCorotBeamModule.jl:144-147 */
enum {
    ORC_BEAM_CONSISTENT_NO_ROT = 0,
    ORC_BEAM_CONSISTENT_WITH_ROT = 1,
    ORC_BEAM_LUMPED_NO_ROT = 2,
    ORC_BEAM_LUMPED_WITH_ROT = 3
};

/* current length; Ft (3x3 column-major) and the natural deformations dN[6] */
double orc_beam_frame(const double *x0, const double *xt, const double *x1x2, const double *RI,
                      const double *RJ, double *Ft, double *dN);

/* One element: x0, u 2x3 node-major, RI, RJ 3x3 column-major, v 2x6
 * node-major (gyroscopic only), sec 10 doubles.  out: 12x12 column-major,
 * or 12 entries for ORC_BEAM_RESTORING. */
int orc_beam_element(int which, const double *x0, const double *u, const double *RI,
                     const double *RJ, const double *v, const double *sec, double E, double nu,
                     double rho, int mass_type, double *out);
int orc_beam_distribload(const double *x0, const double *u, const double *RI, const double *RJ,
                         const double *sec, const double *q, double *out);

/* All elements, global arrays in Julia layouts: xyz, u1 nnodes x 3; R1
 * nnodes x 9 (R[:] per node); v1 nnodes x 6 (may be NULL); sections
 * nelem x 10 row per element; q nelem x 3 row per element (distributed load
 * only).  out: nelem x 144 or nelem x 12. */
int orc_beam_all(int which, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                 const double *u1, const double *R1, const double *v1, const double *sections,
                 double E, double nu, double rho, int mass_type, const double *q, double *out);

void orc_assemble_vector(int64_t nnodes, int64_t nelem, int nen, const int64_t *conn,
                         const int64_t *dofnums, int64_t n, const double *Fe, double *F);

#ifdef __cplusplus
}
#endif
#endif

/*
 * CPU oracle for the shell element-assembly hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * (FinEtoolsFlexStructures.jl 3.6.4) element loops and of the FinEtools
 * assembler semantics.  It is the checker for the CUDA library and the timed
 * CPU baseline; the product never links it.
 *
 * It follows the reference's own dense formulation (explicit 18x18 / 24x24
 * transformation matrices and Q^T E Q congruences) so that it is an
 * independent check of the structure-aware GPU kernels.
 *
 * Conventions (Julia's): xyz is nnodes x 3 column-major; dofnums nnodes x 6
 * column-major, 1-based; conn is nelem x nen row-per-element, 1-based.
 * Element matrices are column-major.
 */
#ifndef FLEXSHELL_ORACLE_H
#define FLEXSHELL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_T3FF = 0, ORC_T3FFCOMP = 1, ORC_Q4RS = 2, ORC_Q4RSCOMP = 3 };
enum { ORC_KEEP_ZEROS = 0, ORC_DROP_ZEROS = 1, ORC_DIAG = 2 };

/* Per-element constitutive data for the layered variants and the
 * homogeneous material.  Group g owns A,B,D (3x3), H (2x2), csmat (3x3),
 * thickness, mass and rotary-inertia densities, all column-major. */
typedef struct {
    int etype;
    /* homogeneous material */
    double Dps[9];
    double Dt[4];
    double rho;
    /* per-element thickness (homogeneous) */
    const double *thickness;     /* nelem */
    /* layup groups (composite) */
    int ngroups;
    const int32_t *group;        /* nelem, 0-based group of each element */
    const double *gA, *gB, *gD;  /* ngroups x 9 */
    const double *gH;            /* ngroups x 4 */
    const double *gcsmat;        /* ngroups x 9 */
    const double *gthick;        /* ngroups */
    const double *gmass;         /* ngroups: mass density per unit area */
    const double *gmoi;          /* ngroups: rotary inertia density */
    /* formulation knobs */
    double stab_c;               /* stab_fun(t,h) = t^2/(t^2 + stab_c h^2) */
    double drill_scale;
    int tsf;                     /* T3: 0 = average B, 1 = average K */
} orc_params;

int orc_normals(int etype, int64_t nnodes, const double *xyz, int64_t nelem,
                const int64_t *conn, const int64_t *order, double threshold_deg,
                const orc_params *p, double *normals, uint8_t *valid);

/* Normals with a built-in material csys kind instead of the isoparametric
 * one: ORC_CSYS_CARTESIAN (params: 3x3 column-major matrix), _CYLINDRICAL
 * (a point on the axis, the unit axis direction), _SPHERICAL (the centre). */
enum { ORC_CSYS_ISOPARAMETRIC = 0, ORC_CSYS_CARTESIAN = 1, ORC_CSYS_CYLINDRICAL = 2, ORC_CSYS_SPHERICAL = 3 };
int orc_normals_csys(int etype, int64_t nnodes, const double *xyz, int64_t nelem,
                     const int64_t *conn, const int64_t *order, double threshold_deg,
                     const orc_params *p, int kind, const double *params, double *normals,
                     uint8_t *valid);

int orc_element_stiffness(const orc_params *p, int64_t e, const double *X,
                          const double *nrm, const uint8_t *nvalid, double *Ke);

int orc_element_mass(const orc_params *p, int64_t e, const double *X, double *tm,
                     double *rm);

/* Element loop + assembly.  `order` (may be NULL) is the sequence in which
 * elements are assembled (layup-group order).  The result is kept in a
 * handle and copied out with orc_result_copy (CSC == CSR arrays for a
 * symmetric matrix; 1-based). */
typedef struct orc_result orc_result;
int orc_assemble(int what /*0 K, 1 M*/, int mode, int64_t nnodes, const double *xyz,
                 int64_t nelem, const int64_t *conn, const int64_t *order,
                 const int64_t *dofnums, int64_t n, const double *normals,
                 const uint8_t *valid, const orc_params *p, int nthreads,
                 orc_result **out);
/* The same assembly of given element matrices (nelem x (6 nen)^2, column-major
 * each), e.g. those of the beam oracle. */
int orc_assemble_elmats(int mode, int nen, int64_t nnodes, int64_t nelem, const int64_t *conn,
                        const int64_t *order, const int64_t *dofnums, int64_t n, const double *Ke,
                        orc_result **out);
int64_t orc_result_nnz(const orc_result *r);
int64_t orc_result_n(const orc_result *r);
void orc_result_copy(const orc_result *r, int64_t *colptr, int64_t *rowval, double *nzval);
void orc_result_free(orc_result *r);

/* Dense element matrices for all elements (column-major ndof x ndof each). */
/* element stiffness matrices summed into the values of a given 1-based CSC
 * pattern (meshes too large for a COO buffer); see the definition */
int orc_csc_accumulate_stiffness(int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                                 const double *normals, const uint8_t *valid, const orc_params *p,
                                 const int64_t *dofnums, int64_t n, const int64_t *colptr,
                                 const int64_t *rowval, double *vals, uint8_t *touched, int64_t *missing,
                                 int nthreads);
int orc_all_element_stiffness(int64_t nnodes, const double *xyz, int64_t nelem,
                              const int64_t *conn, const double *normals,
                              const uint8_t *valid, const orc_params *p, int nthreads,
                              double *Ke_all);

/* Central-difference loop of the reference explicit examples (mass
 * proportional damping, CSR stiffness, zero external force). */
int orc_cd_steps(int64_t n, const int64_t *rowptr, const int64_t *colidx,
                 const double *vals, const double *invMC, const double *C, double dt,
                 int64_t nsteps, double *U, double *V, double *A, int nthreads);

/* Stress resultants at the integration points of the homogeneous shells
 * (inspectintegpoints, src/FEMMShellT3FFModule.jl:850-962: the centroid of a
 * T3FF element; src/FEMMShellQ4RSModule.jl:1061-1170: the four Gauss points
 * of a Q4RS element): quantity ORC_RES_MOMENT (m_xx, m_yy, m_xy),
 * ORC_RES_SHEAR (q_x, q_y, 0), ORC_RES_MEMBRANE (n_xx, n_yy, n_xy) in the
 * output csys.  u: nnodes x 6 column-major displacements and rotations;
 * cs: one 3x3 column-major csys matrix (ncs = 1), one per point (ncs =
 * number of points), or NULL with ncs = 0 for the element frame at each
 * point (the shells' default mcsys, whose updater is _e_g!); out: 3 values
 * per point, points in element order. */
enum { ORC_RES_MOMENT = 1, ORC_RES_SHEAR = 2, ORC_RES_MEMBRANE = 3 };
int orc_resultants(int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                   const double *normals, const uint8_t *valid, const orc_params *p,
                   const double *u, int quant, const double *cs, int64_t ncs, double *out);

/* The same loop with the external force F(t) = g(t) Fmag of the example's
 * force!: mul[k] = g(k dt) (zero from k = nmul), the state at step index
 * step0 (t = step0 dt). */
int orc_cd_steps_load(int64_t n, const int64_t *rowptr, const int64_t *colidx,
                      const double *vals, const double *invMC, const double *C, double dt,
                      int64_t nsteps, double *U, double *V, double *A, const double *Fmag,
                      const double *mul, int64_t nmul, int64_t step0, int nthreads);

/* Distributed loads, distribloads(FEMMBase(IntegDomain(fes, rule)), geom, P,
 * ForceIntensity, m) of FinEtools 8.2.5 on an L2 (nen 2, GaussRule(1, order
 * 1..3), m 1..3: boundary curves of a shell mesh), T3 (nen 3, TriRule npts
 * 1, 3, 6) or Q4 (nen 4, GaussRule(2, order 1..3), m 2 or 3) element set: force 6
 * values per entry, nforce 1, nelem or nelem x npoints; F (n) accumulated in
 * element order; dofnums nnodes x 6 column-major, 1-based. */
int orc_distribloads(int nen, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                     const int64_t *dofnums, int rule, int m, const double *force, int64_t nforce, int64_t n,
                     double *F);
/* The rule's points, element order, 9 values each: location, x_xi, x_eta
 * (x_eta zero for the line element). */
int orc_integration_points(int nen, int64_t nnodes, const double *xyz, int64_t nelem, const int64_t *conn,
                           int rule, double *out);

/* Laminate stiffness of a layup (CompositeLayupModule). */
int orc_laminate(int nplies, const double *ply_Dps, const double *ply_Dts,
                 const double *ply_t, const double *ply_angle_deg, const double *ply_rho,
                 double offset, int shear_model /*0 VS, 1 constant*/, double tcf,
                 double *A, double *B, double *D, double *H, double *mass_density,
                 double *moi_density);

#ifdef __cplusplus
}
#endif
#endif

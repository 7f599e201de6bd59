/*
 * flexshell: GB300 (sm_103a) shell element assembly -- C ABI.
 *
 * Drop-in boundary for the element-assembly hot path of
 * FinEtoolsFlexStructures.jl 3.6.4.  Every entry point is plain C (pointers
 * and sizes, no framework types) so that the Julia shim can `ccall` it; the
 * Julia methods keep the reference signatures and return the same
 * SparseMatrixCSC{Float64,Int64}.
 *
 * Layouts follow Julia: geometry `nnodes x 3` column-major, dof numbers
 * `nnodes x 6` column-major and 1-based (free dofs first, as numberdofs!),
 * connectivity one row of `nen` 1-based node numbers per element
 * (reinterpret(Int, fes.conn)).  Matrices come back as 1-based CSC arrays;
 * the assembled matrices are symmetric, so they are also the CSR arrays.
 *
 * Every function returns FS_OK (0) or an FS_ERR_* code; fs_last_error()
 * gives the message.  Calls are blocking (the context stream is
 * synchronised before return) except where noted.  A context is used by
 * one host thread at a time.
 */
#ifndef FLEXSHELL_H
#define FLEXSHELL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FS_OK 0
#define FS_ERR_BAD_INPUT 1        /* invalid argument or mesh data            */
#define FS_ERR_CUDA 2             /* CUDA runtime error                       */
#define FS_ERR_OOM 3              /* device allocation failed                 */
#define FS_ERR_SINGULAR_METRIC 4  /* Q4: "Singular metric matrix" (src/FEMMShellQ4RSModule.jl:308-311) */
#define FS_ERR_UNSUPPORTED 5      /* option outside the supported family      */
#define FS_ERR_STATE 6            /* call order (e.g. no associategeometry!)  */
#define FS_ERR_TIMEOUT 7          /* bounded device wait expired              */

/* element families (FEMM types of the reference) */
#define FS_T3FF 0       /* FEMMShellT3FF,     src/FEMMShellT3FFModule.jl     */
#define FS_T3FFCOMP 1   /* FEMMShellT3FFComp, src/FEMMShellT3FFCompModule.jl */
#define FS_Q4RS 2       /* FEMMShellQ4RS,     src/FEMMShellQ4RSModule.jl     */
#define FS_Q4RSCOMP 3   /* FEMMShellQ4RSComp, src/FEMMShellQ4RSCompModule.jl */
#define FS_COROTBEAM 4  /* FEMMCorotBeam (2-node L2 beams), src/FEMMCorotBeamModule.jl */

/* arithmetic of the element strain rows and Gram products */
#define FS_FP64 0       /* everything in double: the drop-in                 */
#define FS_MIXED 1      /* float element arithmetic on element frames and
                           coordinates formed in double (the Q4 Gauss-point
                           frames and drilling factor in float); CSR values
                           summed from the float blocks as float pairs and
                           rounded once to double                            */
#define FS_MIXED_COMP 2 /* as FS_MIXED, with the element Gram products
                           accumulated in compensated float sums (Dot2 for
                           T3's at most 9 rows per entry, three levels for
                           Q4's 33), kept as float pairs and summed into
                           float triples: the stiffness keeps the rigid-body
                           null space to O(eps^2), for thin-plate eigenvalues */

/* assembler semantics (FinEtools assemblers) */
#define FS_ASM_SPARSE 0      /* SysmatAssemblerSparse / SysmatAssemblerSparseCSRSymm
                                (src/AssemblyModule.jl:20-53): union pattern, explicit zeros kept */
#define FS_ASM_SPARSE_SYMM 1 /* SysmatAssemblerSparseSymm (default of stiffness/mass):
                                entries whose assembled value is exactly zero are dropped */
#define FS_ASM_DIAG 2        /* SysmatAssemblerSparseDiag: diagonal only */

typedef struct fs_ctx fs_ctx;

/* Formulation parameters of a homogeneous FEMM (FEMMShellT3FF / FEMMShellQ4RS fields,
 * src/FEMMShellT3FFModule.jl:101-112, src/FEMMShellQ4RSModule.jl:69-79). */
typedef struct {
    int32_t transv_shear_formulation; /* T3FF only: 0 average B (default), 1 average K */
    int32_t reserved;
    double drilling_stiffness_scale;  /* default 1.0 */
    double threshold_angle;           /* degrees, default 30.0 */
    double stab_c;                    /* stab_fun(t,h) = t^2/(t^2 + stab_c*h^2):
                                         T3FF default 5/12/1.5, Q4RS default 0.1 */
    double Dps[9];                    /* plane-stress stiffness, column-major 3x3 */
    double Dt[4];                     /* transverse-shear stiffness, column-major 2x2
                                         (the element applies the 5/6 factor)     */
    double rho;                       /* mass density                              */
    double thickness;                 /* used when no per-element thickness given  */
} fs_shell_params;

/* One layup group (CompositeLayup of src/CompositeLayupModule.jl:185-225,
 * reduced on the host with laminate_stiffnesses!, laminate_transverse_stiffness!
 * and laminate_inertia!, or with fs_laminate below). */
typedef struct {
    double A[9], B[9], D[9]; /* column-major 3x3 */
    double H[4];             /* column-major 2x2 */
    double csmat[9];         /* layup coordinate system (columns = basis vectors) */
    double thickness;        /* thickness(layup) */
    double mass_density;     /* laminate_inertia! first result  */
    double moi_density;      /* laminate_inertia! second result */
} fs_layup_group;

/* --- context ------------------------------------------------------------- */
int fs_ctx_create(int device, fs_ctx **out);
int fs_ctx_destroy(fs_ctx *ctx);
/* Copies the last error message of this context (NUL terminated). */
int fs_last_error(const fs_ctx *ctx, char *buf, size_t len);
/* The CUDA stream (cudaStream_t) all work of the context runs on. */
int fs_stream(const fs_ctx *ctx, void **stream);

/* --- inputs --------------------------------------------------------------- */
/* Mesh, connectivity and dof numbering (fes.conn, geom0.values, dchi.dofnums).
 * `order` (may be NULL) is the 1-based sequence in which elements are
 * assembled; the layered FEMMs assemble layup group by layup group
 * (src/FEMMShellT3FFCompModule.jl:600-606).  `dofnums` may be NULL and set
 * later with fs_dofs_set.  Uploads the arrays. */
int fs_mesh_set(fs_ctx *ctx, int elem_type, int64_t nnodes, const double *xyz, int64_t nelem,
                const int64_t *conn, const int64_t *order, const int64_t *dofnums);
/* New geometry for the same connectivity (geom0.values); keeps normals and pattern. */
int fs_geometry_set(fs_ctx *ctx, const double *xyz);
/* Dof numbering (dchi.dofnums after numberdofs!), nnodes x 6 column-major, 1-based. */
int fs_dofs_set(fs_ctx *ctx, const int64_t *dofnums);
/* Parameters; `thickness` (may be NULL) is per element, in mesh order. */
int fs_params_set(fs_ctx *ctx, const fs_shell_params *params, const double *thickness);
/* Layup groups of a layered FEMM; `elem_group` is the 0-based group of each element. */
int fs_layups_set(fs_ctx *ctx, int32_t ngroups, const fs_layup_group *groups,
                  const int32_t *elem_group);

/* --- associategeometry! ----------------------------------------------------- */
/* Nodal normals and validity flags with the default (isoparametric) normals,
 * or the layup csys third axis for the layered FEMMs
 * (src/FEMMShellT3FFModule.jl:570-616, src/FEMMShellQ4RSModule.jl:472-525). */
int fs_normals_compute(fs_ctx *ctx);
/* The same with a built-in material csys (the FEMM's mcsys) in place of the
 * isoparametric one (_compute_nodal_normal!, src/FEMMShellT3FFModule.jl:226-230,
 * in associategeometry! :570-616 / src/FEMMShellQ4RSModule.jl:472-525): the
 * kinds the reference examples define as closures, generalised.
 *   FS_CSYS_CARTESIAN   params[9]: the 3x3 column-major csys matrix (its third
 *                       column is the normal; bent_strip_examples.jl:15-20)
 *   FS_CSYS_CYLINDRICAL params[6]: a point on the axis and the unit axis
 *                       direction (radial normal; cylindrical! of
 *                       clamp_cyl_expl_examples.jl:61-67 is point 0, axis y)
 *   FS_CSYS_SPHERICAL   params[3]: the centre (radial normal; spherical! of
 *                       hemisphere_examples.jl:31-39 is the origin)
 * Homogeneous shells only (layered ones use their layup csys). */
#define FS_CSYS_ISOPARAMETRIC 0
#define FS_CSYS_CARTESIAN 1
#define FS_CSYS_CYLINDRICAL 2
#define FS_CSYS_SPHERICAL 3
int fs_normals_compute_csys(fs_ctx *ctx, int kind, const double *params);
/* Normals computed by the caller (e.g. a user `mcsys`), nnodes x 3 column-major. */
int fs_normals_set(fs_ctx *ctx, const double *normals, const uint8_t *valid);
int fs_normals_get(fs_ctx *ctx, double *normals, uint8_t *valid);

/* --- stiffness / mass ------------------------------------------------------- */
/* stiffness(femm, assembler, geom0, u1, Rfield1, dchi)
 * (src/FEMMShellT3FFModule.jl:635-736, src/FEMMShellQ4RSModule.jl:877-947 and the
 * layered variants).  `nrows` is the matrix size (nalldofs(dchi), or nfreedofs for
 * the free block); dofs above it are left out as FinEtools does.  The sparsity
 * pattern is built on the first call for a mesh and reused.  The matrix stays
 * on the device until fs_matrix_copy. */
int fs_stiffness(fs_ctx *ctx, int precision, int assembler, int64_t nrows, int64_t *nnz_out);
/* mass(femm, assembler, geom0, dchi): the lumped mass
 * (src/FEMMShellT3FFModule.jl:757-811, src/FEMMShellQ4RSModule.jl:968-1022). */
int fs_mass(fs_ctx *ctx, int assembler, int64_t nrows, int64_t *nnz_out);
/* The matrix of the last fs_stiffness / fs_mass call into caller memory:
 * colptr[nrows+1], rowval[nnz], nzval[nnz], 1-based CSC.  Any pointer may be NULL. */
int fs_matrix_copy(fs_ctx *ctx, int64_t *colptr, int64_t *rowval, double *nzval);
/* Two-phase stiffness into host arrays for the pattern-keeping assembler
 * (FS_ASM_SPARSE, also the FF block with nrows = nfreedofs): fs_pattern builds
 * (or reuses) the pattern for `nrows` and returns the number of stored entries,
 * so that the caller can allocate colptr[nrows+1], rowval[nnz], nzval[nnz];
 * fs_stiffness_copy then assembles the values and fills the three arrays
 * (1-based CSC == CSR), the pattern copy running on a second stream while the
 * element and gather kernels run.  Results equal fs_stiffness + fs_matrix_copy. */
int fs_pattern(fs_ctx *ctx, int64_t nrows, int64_t *nnz_out);
int fs_stiffness_copy(fs_ctx *ctx, int precision, int64_t nrows, int64_t *colptr, int64_t *rowval,
                      double *nzval);
/* Device pointers of the last matrix (0-based CSR; valid until the next call). */
int fs_matrix_device(fs_ctx *ctx, const int64_t **rowptr, const int32_t **colidx,
                     const double **vals, int64_t *nrows, int64_t *nnz);
/* Device times (milliseconds, CUDA events on the context stream) of the last
 * fs_stiffness call: [0] element kernel, [1] CSR gather, [2] symbolic phase of
 * the last pattern build, [3] zero compaction.  `n` entries are written. */
int fs_timings(const fs_ctx *ctx, double *out, int n);
/* Tile-shape autotuner of the shell assembly (elements per block of the
 * element kernel; warps per block of the CSR gather and whether each
 * node-block pair is summed once, by the lower node, and copied transposed
 * into the upper node's rows, or by both nodes).  Mode 1 (the default;
 * environment FLEXSHELL_AUTOTUNE=0 makes 0 the default): the first fs_stiffness
 * call for a new key (element family, precision, average-K option, log2 of the
 * element count; meshes of at least 4096 elements) times every candidate on the
 * context's mesh and the choice is reused by the whole process; 0: built-in
 * shapes (pairs summed once); 2: re-tune on the next call; 3: built-in shapes
 * with every pair summed by both nodes.  No choice changes the results. */
int fs_autotune(fs_ctx *ctx, int mode);
/* Shapes used by the last fs_stiffness: out[0] elements per block (0 =
 * default), out[1] gather warps per block (0 = default), out[2] 1 if tuned. */
int fs_tuning(const fs_ctx *ctx, int32_t *out);
/* The same and the gather's mode: out[0..min(n, 4)) = elements per block,
 * gather warps per block, 1 if tuned, 1 if each node-block pair is summed by
 * one of its two nodes and copied transposed into the other's rows (0: both
 * nodes sum it).  Either mode gives bitwise the same values. */
int fs_tuning_ex(const fs_ctx *ctx, int32_t *out, int n);
/* Allocation-free stiffness values.  No counterpart in the reference: it is for
 * callers that cannot let the library allocate device memory at call time (a
 * host whose own pool allocator owns the device memory, or a solver loop under
 * a fixed memory budget).  It writes the CSR values of the stiffness, in the
 * order of the pattern that fs_stiffness with FS_ASM_SPARSE returns, into the
 * caller's device buffer `vals` (vals_len >= nnz).  The pattern for `nrows`
 * must exist (one fs_stiffness or fs_mass call at set-up).  Element matrices
 * are staged in a fixed 32 MiB device array inside the library, so
 * nelem * 36 nen (nen + 1)/2 * (4 for FS_MIXED, else 8) bytes (the upper
 * node blocks of its element matrices) must fit in it (19,418 T3FF elements in FP64); larger meshes get FS_ERR_UNSUPPORTED.
 * It calls no cudaMalloc/cudaFree.  The array's address is looked up by
 * fs_ctx_create (which therefore loads the library's device code and the
 * array, with 32 MiB free, at context creation); every call shares the one
 * array, so calls that overlap on the GPU race and must be serialised by the
 * caller. */
int fs_stiffness_values_noalloc(fs_ctx *ctx, int precision, int64_t nrows, double *vals,
                                int64_t vals_len);
/* Element matrices in the global basis (nelem x (6 nen)^2, each column-major), in
 * mesh order; for parity checks.  FS_MIXED_COMP entries are float pairs
 * returned as the double nearest hi + lo (a pair can hold more bits than a
 * double when its low half is far below its high half's last place). */
int fs_element_matrices(fs_ctx *ctx, int precision, double *out);
/* Lumped element masses (tmass, rmass) per element, in mesh order. */
int fs_element_masses(fs_ctx *ctx, double *out);

/* --- explicit central difference (examples/.../plate_expl_examples.jl:61-94) --- */
/* Uses the last matrix from fs_stiffness (must be nrows x nrows; FS_ERR_STATE
 * when the last matrix assembled is not a stiffness).  A later assembly in the
 * context (fs_stiffness, fs_mass, fs_beam_matrix, a new fs_pattern) or a new
 * mesh or dof numbering ends the explicit state: fs_explicit_* then return
 * FS_ERR_STATE until fs_explicit_setup is called again.  invMC and C are
 * the per-dof vectors of _cd_loop! (:69-71).  Values are kept in double
 * (precision FS_FP64), rounded to float (FS_MIXED), or as float plus a bf16
 * residual (FS_MIXED_COMP); K U is formed in double (FS_FP64), in float from a
 * float copy of U (FS_MIXED), or in compensated float sums from a float-pair
 * copy of U (FS_MIXED_COMP); the state update is double with Kahan
 * compensation. */
int fs_explicit_setup(fs_ctx *ctx, int precision, const double *invMC, const double *C, double dt);
int fs_explicit_set_state(fs_ctx *ctx, const double *U, const double *V, const double *A);
/* External force of the reference example's force!(F, t): F = g(t) Fmag
 * (plate_expl_examples.jl:202-209 with Fmag from distribloads or a point
 * load), applied in every step as F = g Fmag - (K U + C (V + dt/2 A)).
 * Fmag: n values (system numbering); mul[k] = g(k dt), k = 0..nmul-1 (zero
 * beyond); step0: the step index k of the current state (t = k dt).  The step
 * index advances with every step run.  Fmag = NULL removes the load.  The
 * initial acceleration A = invMC F(0) is the caller's (fs_explicit_set_state). */
int fs_explicit_set_load(fs_ctx *ctx, const double *Fmag, const double *mul, int64_t nmul, int64_t step0);
/* Runs nsteps steps; the step loop is captured once into a CUDA graph. */
int fs_explicit_run(fs_ctx *ctx, int64_t nsteps);
int fs_explicit_get_state(fs_ctx *ctx, double *U, double *V, double *A);
/* Largest angular frequency of (K, M) for a diagonal M (mdiag, nrows entries) by
 * power iteration on the last assembled stiffness (FS_ERR_STATE when the last
 * matrix assembled is not a stiffness): the reference's `pwr`
 * (examples/shells/dynamics/homogeneous/explicit/clamp_cyl_expl_examples.jl:131-142),
 * with a deterministic start vector from `seed`; dt_crit = 2 / omega_max. */
int fs_power_iteration(fs_ctx *ctx, const double *mdiag, int64_t iters, uint64_t seed,
                       double *omega_max);

/* --- shift-invert support for the lowest modes ---------------------------------
 * The inner step of the reference's modal analyses, eigs(K, M; nev, which = :SM)
 * with a shift (ARPACK's shift-invert mode; test/test_shell_dynamics.jl:79-80,
 * test/test_composite_shell_dynamics.jl): fs_shift_factor factorises
 * K - sigma diag(mdiag) on the device, K the last matrix assembled by
 * fs_stiffness (or fs_beam_matrix with FS_BEAM_STIFFNESS) and mdiag its nrows
 * lumped masses (fs_mass with FS_ASM_DIAG, assembled before the stiffness).
 * The factor is a banded Cholesky factor in double; its half-bandwidth comes
 * from the dof numbering (returned in *bandwidth_out) and its storage is
 * nrows x (bandwidth + 512) doubles (more than 160 GiB: FS_ERR_UNSUPPORTED).
 * A matrix that is not positive definite gives FS_ERR_BAD_INPUT.
 * fs_shift_solve solves (K - sigma M) X = B for nrhs host right-hand sides
 * (nrows x nrhs, column-major).  A new mesh or dof numbering (fs_mesh_set,
 * fs_dofs_set) releases the factor: fs_shift_solve then returns FS_ERR_STATE
 * until fs_shift_factor is called again.  An eigensolver (ARPACK) supplies
 * the rest. */
int fs_shift_factor(fs_ctx *ctx, double sigma, const double *mdiag, int64_t *bandwidth_out);
int fs_shift_solve(fs_ctx *ctx, int nrhs, const double *b, double *x);

/* --- co-rotational beams (src/FEMMCorotBeamModule.jl) ---------------------------
 * Mesh: fs_mesh_set with FS_COROTBEAM, conn nelem x 2.  All beam arithmetic is
 * double.  The matrices are assembled like the shell matrices (same assemblers,
 * same CSR/CSC output through fs_matrix_copy); the vectors are summed in element
 * order (SysvecAssembler). */

/* what fs_beam_matrix assembles */
#define FS_BEAM_STIFFNESS 0    /* stiffness(femm, assembler, geom0, u1, Rfield1, dchi)  :972-1023  */
#define FS_BEAM_GEOSTIFFNESS 1 /* geostiffness(femm, assembler, geom0, u1, Rfield1, dchi) :1042-1094 */
#define FS_BEAM_MASS 2         /* mass(femm, assembler, geom0, u1, Rfield1, dchi; mass_type) :810-862 */
#define FS_BEAM_GYROSCOPIC 3   /* gyroscopic(femm, assembler, geom0, u1, Rfield1, v1, dchi; mass_type) :883-952 */

/* mass_type (MASS_TYPE_* of src/FEMMCorotBeamModule.jl:144-147) */
#define FS_BEAM_MASS_CONSISTENT_NO_ROTATION_INERTIA 0
#define FS_BEAM_MASS_CONSISTENT_WITH_ROTATION_INERTIA 1 /* the reference default */
#define FS_BEAM_MASS_LUMPED_DIAGONAL_NO_ROTATION_INERTIA 2
#define FS_BEAM_MASS_LUMPED_DIAGONAL_WITH_ROTATION_INERTIA 3

/* Cross-section of one element: the FESetL2Beam fields A, I1, I2, I3, J, A2s,
 * A3s (INFINITY for a Bernoulli section) and x1x2_vector
 * (src/FESetL2BeamModule.jl:20-31). */
typedef struct {
    double A, I1, I2, I3, J, A2s, A3s;
    double x1x2_vector[3];
} fs_beam_section;

/* Sections (nelem, mesh order) and the MatDeforElastIso constants. */
int fs_beam_setup(fs_ctx *ctx, const fs_beam_section *sections, double E, double nu, double rho);
/* Configuration of the next calls: u1 (nnodes x 3), Rfield1 (nnodes x 9, the
 * column-major rotation matrix R[:] of each node, as Rfield1.values) and the
 * velocities v1 (nnodes x 6, gyroscopic only), all column-major.  A NULL array
 * means zero displacement, identity rotations, zero velocity. */
int fs_beam_state_set(fs_ctx *ctx, const double *u1, const double *Rfield1, const double *v1);
/* Assemble FS_BEAM_STIFFNESS / GEOSTIFFNESS / MASS / GYROSCOPIC (nrows as for
 * fs_stiffness; mass_type used by MASS and GYROSCOPIC).  Copy out with
 * fs_matrix_copy. */
int fs_beam_matrix(fs_ctx *ctx, int which, int mass_type, int assembler, int64_t nrows, int64_t *nnz_out);
/* restoringforce(femm, assembler, geom0, u1, Rfield1, dchi) (:1112-1159) into
 * host F[nrows]; dofs above nrows are left out. */
int fs_beam_restoringforce(fs_ctx *ctx, int64_t nrows, double *F);
/* distribloads_global(femm, assembler, geom0, u1, Rfield1, dchi, fi)
 * (:1186-1247): force per unit length in global components, one 3-vector for
 * all elements (per_element 0) or one per element (nelem x 3, row per element). */
int fs_beam_distribloads_global(fs_ctx *ctx, const double *q, int per_element, int64_t nrows, double *F);
/* Element matrices (nelem x 144, column-major each, mesh order) or element
 * vectors (which 4 = restoring force, 5 = distributed load with q as above;
 * nelem x 12), for parity checks. */
int fs_beam_element_matrices(fs_ctx *ctx, int which, int mass_type, double *out);
int fs_beam_element_vectors(fs_ctx *ctx, int which, const double *q, int per_element, double *out);

/* --- batched assembly of uneven meshes -------------------------------------
 * Several homogeneous meshes of one family (FS_T3FF or FS_Q4RS) with the
 * parameters of the last fs_params_set (whose thickness is replaced by one
 * thickness per mesh).  Mesh i has nnodes[i] nodes (xyz[i], nnodes x 3
 * column-major), nelem[i] elements (conn[i], 1-based within the mesh), its dof
 * numbers (dofnums[i], nnodes x 6, 1-based within the mesh) and matrix size
 * nrows[i].  The meshes are assembled together: one element-kernel launch over
 * the work-list of all their elements and one gather launch over all their
 * nodes; each mesh's matrix is bitwise the one fs_stiffness gives for it
 * alone.  fs_batch_set computes the default normals. */
int fs_batch_set(fs_ctx *ctx, int elem_type, int32_t nmeshes, const int64_t *nnodes, const double *const *xyz,
                 const int64_t *nelem, const int64_t *const *conn, const int64_t *const *dofnums,
                 const int64_t *nrows, const double *thickness);
/* Assemble all meshes' stiffness matrices; nnz_out[i] (may be NULL) = stored
 * entries of mesh i. */
int fs_batch_stiffness(fs_ctx *ctx, int precision, int assembler, int64_t *nnz_out);
/* Mesh i's matrix of the last fs_batch_stiffness: 1-based CSC (== CSR)
 * colptr[nrows[i]+1], rowval[nnz_out[i]], nzval[nnz_out[i]].  FS_ERR_STATE
 * when another matrix (a mass, another size) has been assembled since. */
int fs_batch_matrix_copy(fs_ctx *ctx, int32_t mesh, int64_t *colptr, int64_t *rowval, double *nzval);

/* Restoring force -K U of the shells for the generalized displacements U
 * (mat_n entries, system numbering) with the last matrix assembled by
 * fs_stiffness (FS_ERR_STATE when the last matrix is not a stiffness); F gets
 * mat_n entries.  The reference shells have no such
 * function: _cd_loop! (plate_expl_examples.jl:85) subtracts E = K U; the sign
 * here follows FEMMCorotBeam.restoringforce (force on the nodes). */
int fs_restoring_force(fs_ctx *ctx, const double *U, double *F);

/* Stress resultants at the integration points of a homogeneous shell mesh,
 * in double: inspectintegpoints(femm, geom0, u, felist, inspector, idat,
 * quantity; outputcsys) of FEMMShellT3FF (src/FEMMShellT3FFModule.jl:850-962,
 * one point per element: the centroid) and FEMMShellQ4RS
 * (src/FEMMShellQ4RSModule.jl:1061-1170, the four Gauss points in the
 * reference's order), for all elements at once; the host applies the
 * inspector to the points of felist.  quantity: FS_RES_MOMENT (:bending,
 * :moment, :bending_moment -> m_xx, m_yy, m_xy), FS_RES_SHEAR (:shear,
 * :transverse, :transverse_shear -> q_x, q_y, 0), FS_RES_MEMBRANE (:membrane,
 * :membrane_force -> n_xx, n_yy, n_xy), in the output csys.
 * u: nnodes x 6 column-major (u.values); csmat: the output csys, ncs = 1 one
 * 3x3 column-major matrix for every point, or ncs = number of points (nelem
 * for T3FF, 4 nelem for Q4RS), one per point in element order, or csmat =
 * NULL with ncs = 0: the element frame at each point (the shells' default
 * mcsys, isoparametric! = _e_g!); out: 3 doubles per point, element order.
 * Needs the normals (associategeometry!). */
#define FS_RES_MOMENT 1
#define FS_RES_SHEAR 2
#define FS_RES_MEMBRANE 3
int fs_resultants(fs_ctx *ctx, int quantity, const double *u, const double *csmat, int64_t ncs, double *out);

/* Distributed loads on a shell mesh or on its boundary curves:
 * distribloads(FEMMBase(IntegDomain(fes, rule)), geom0, dchi, fi, m) of
 * FinEtools 8.2.5, as the reference calls it on its shell element sets
 * (examples/shells/dynamics/homogeneous/explicit/plate_expl_examples.jl:196-199,
 * test/test_shell_statics.jl:84-86) and on the L2 edges of meshboundary
 * (test/test_shell_statics.jl:212-215, test/test_composite_shell_statics.jl:80-88).
 * The element set is the context's mesh: T3 (FS_T3FF) with TriRule(npts),
 * npts 1, 3 or 6; Q4 (FS_Q4RS) with GaussRule(2, order), order 1, 2 or 3;
 * two-node line elements (FS_COROTBEAM) with GaussRule(1, order), order 1, 2
 * or 3.  m: 2 or 3 on surfaces, 1, 2 or 3 on lines (the element's other
 * dimension is 1).  force: the ForceIntensity's six
 * components, nforce = 1 (uniform), nelem (one per element, element order) or
 * nelem x npoints (one per integration point, the points of
 * fs_integration_points).  F: nrows entries (nalldofs, or nfreedofs for
 * SysvecAssemblerFBlock), dofs above nrows dropped.  No parameters needed. */
int fs_distribloads(fs_ctx *ctx, int rule, int m, const double *force, int64_t nforce, int64_t nrows, double *F);

/* The integration points of the same rules, element order, nine doubles per
 * point: the location and the two parent tangents x,xi and x,eta (the
 * arguments the reference's ForceIntensity callback receives as XYZ and
 * tangents; x,eta is zero on a line element, whose callback gets x,xi only). */
int fs_integration_points(fs_ctx *ctx, int rule, double *out);

/* --- layup reduction (src/CompositeLayupModule.jl:246-330) ------------------ */
/* ply_Dps: nplies x 9, ply_Dts: nplies x 4 (column-major each); angles in degrees;
 * shear_model 0 = Vinson-Sierakowski, 1 = constant `tcf`. Host only. */
int fs_laminate(int32_t nplies, const double *ply_Dps, const double *ply_Dts,
                const double *ply_thickness, const double *ply_angle_deg, const double *ply_rho,
                double offset, int32_t shear_model, double tcf, fs_layup_group *out);

#ifdef __cplusplus
}
#endif
#endif

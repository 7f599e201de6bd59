// Internal declarations of the flexshell CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/flexshell.h"
#include "fs_elem_math.cuh"
#include "fs_beam_math.cuh"

namespace fs {

// Device arrays owned by a context.  Sizes are in elements.
template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
};

// Status bits written by kernels (never trapping; the host turns them into codes).
enum : int {
    DEV_OK = 0,
    DEV_BAD_CONN = 1,
    DEV_BAD_DOF = 2,
    DEV_SINGULAR = 4,
    DEV_VALENCE = 8,     // too many elements at one node
    DEV_NEIGHBORS = 16,  // too many neighbour nodes
    DEV_BAD_ORDER = 32,
    DEV_NEG_DRILL = 64,
};

static const int MAX_PAIRS_PER_NODE = 64;   // elements meeting at one node

// Element matrices are stored as their upper 6x6 node blocks (a <= b) only,
// row-major inside a block; ub(a, b) is the block's position.
__host__ __device__ __forceinline__ int n_upper_blocks(int nen) { return nen * (nen + 1) / 2; }
__host__ __device__ __forceinline__ int ub(int a, int b, int nen) { return a * nen - a * (a - 1) / 2 + (b - a); }
static const int MAX_NBRS = 255;            // neighbour nodes of one node (slots are 8-bit)

struct MeshDev {
    int etype = -1, nen = 0;
    int64_t nnodes = 0, nelem = 0;
    double *xyz = nullptr;       // 3 x nnodes (SoA, Julia column-major)
    int32_t *conn = nullptr;     // nelem x nen, by assembly rank, 0-based
    int32_t *elem_of_rank = nullptr;  // rank -> mesh element
    int32_t *dof = nullptr;      // 6 x nnodes (SoA), 1-based as given
    double *thick = nullptr;     // per rank
    int32_t *group = nullptr;    // per rank
    GroupConst *groups = nullptr;
    int ngroups = 0;
    double *normals = nullptr;   // 3 x nnodes
    float *normals_f = nullptr;  // the same rounded to float (the float rows' triads)
    uint8_t *valid = nullptr;
    // node -> (element rank, local node) adjacency, ascending rank
    int64_t npairs = 0;
    int64_t *pp = nullptr;       // nnodes + 1
    int32_t *pair_e = nullptr;   // rank << 2 | local node
    int32_t *elem_pair = nullptr;  // per rank x nen: pair index
};

struct PatternDev {
    int64_t n = -1;              // matrix size the pattern is built for
    int64_t nnz = 0;
    int maxlen = 0;              // longest row
    int64_t *nbr_off = nullptr;  // nnodes + 1
    int32_t *nbr = nullptr;      // neighbour nodes, sorted
    uint32_t *pair_slots = nullptr;  // per pair: 8-bit slot of each element node
    int16_t *colpos = nullptr;   // per node: 6 x nnbr positions in the row (or -1)
    uint16_t *colsrc = nullptr;  // per node: for row position j, neighbour slot * 6 + component
    // per (node, neighbour slot): the node's contributions to that slot's columns, in
    // ascending pair order; an entry is q | b << 6 | (b < a_q) << 8 with q the pair
    // index within the node (< 64), b the element node at that slot, a_q the node's
    // own element node (the block is the mirror of an upper block when b < a_q).
    // The entries of node r start at pp[r] * nen; sl_off gives each slot's start.
    uint16_t *sl_off = nullptr;  // per (node, slot), relative to the node's first entry
    uint16_t *sl_ent = nullptr;  // npairs * nen
    int32_t *rowlen = nullptr;   // per node: row length L
    // per (node, slot): node-block pairs summed once (k_slot_mirror); sym false
    // when the neighbour entry indices would not fit 28 bits (every node sums
    // its own rows)
    uint32_t *sl_mir = nullptr;
    int32_t *lc = nullptr;       // per node: row positions summed with pairs summed once (rows <= 64)
    int maxlc = 0;               // longest of those (the longest row without sym)
    bool sym = false;
    int64_t *rowptr = nullptr;   // n + 1
    int32_t *colidx = nullptr;   // nnz, 0-based
    int64_t *diag_rowptr = nullptr;  // diagonal pattern (n + 1)
    int32_t *diag_colidx = nullptr;  // n
    int64_t *tmp_cnt = nullptr;      // temporaries of the symbolic phase
    int32_t *tmp_owner = nullptr;
    // allocated capacities (elements): a rebuild reuses the buffers that fit
    size_t cap_nbr_off = 0, cap_nbr = 0, cap_pair_slots = 0, cap_colpos = 0, cap_colsrc = 0, cap_rowlen = 0,
           cap_sl_off = 0, cap_sl_ent = 0, cap_rowptr = 0, cap_colidx = 0, cap_diag_rowptr = 0,
           cap_diag_colidx = 0, cap_tmp_cnt = 0, cap_tmp_owner = 0, cap_sl_mir = 0, cap_lc = 0;
};

}  // namespace fs

struct fs_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host copies overlapping the kernels (fs_stiffness_copy)
    cudaEvent_t copy_ev[2] = {nullptr, nullptr};
    std::string err;
    int *d_status = nullptr;     // kernel status bits
    fs::MeshDev mesh;
    fs_shell_params params{};
    fs::MatConst mc{};
    bool params_set = false;
    bool normals_ready = false;
    bool dofs_ready = false;
    fs::PatternDev pat;
    // element matrices (block layout), element masses
    void *ke = nullptr;
    size_t ke_bytes = 0;
    double *tmrm = nullptr;
    // current matrix; mat_kind 0 a stiffness (shell or beam), 1 a mass, 2
    // another beam matrix
    int mat_kind = -1;
    int64_t mat_n = 0, mat_nnz = 0;
    const int64_t *mat_rowptr = nullptr;
    const int32_t *mat_colidx = nullptr;
    double *vals = nullptr;
    size_t vals_cap = 0;
    // compacted pattern (assembler dropping zeros)
    int64_t *cmp_rowptr = nullptr;
    int32_t *cmp_colidx = nullptr;
    double *cmp_vals = nullptr;
    size_t cmp_cap = 0;
    // phase timing events: element start/end, gather end, compaction end
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double t_symbolic_ms = 0.0;
    double t_compact_ms = 0.0;
    bool timed = false;
    // scratch
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // device address of the allocation-free path's fixed scratch array
    // (fs_noalloc.cu) and the error of its lookup, if it failed
    void *noalloc_scratch = nullptr;
    std::string noalloc_err;
    // banded Cholesky factor of K - sigma M (fs_eigen.cu), opaque here
    void *shift = nullptr;
    // staging for host copies
    int64_t *stage64 = nullptr;
    size_t stage_cap = 0;
    // host copies re-applied when the mesh changes
    std::vector<double> h_thickness;
    std::vector<fs_layup_group> h_groups;
    std::vector<int32_t> h_egroup;
    // explicit dynamics
    struct Explicit {
        int precision = 0;
        int64_t n = 0;
        double dt = 0;
        double *U = nullptr, *V = nullptr, *A = nullptr, *F = nullptr;
        double *cU = nullptr, *cV = nullptr;  // Kahan compensations
        double *invMC = nullptr, *C = nullptr;
        float *vals32 = nullptr;
        float *U32 = nullptr;  // float copy of U read by the float restoring force
        // 6x6 node-block form of K (block rows = the pattern's neighbour lists)
        bool bsr = false;
        int64_t nnodes = 0;
        void *blk = nullptr;          // nbr_total x 36 (float or double)
        void *res = nullptr;          // FS_MIXED_COMP: the rounding residual of the float
                                      // values (K - float(K)) in bf16, same layout as blk
                                      // (block form) or vals32 (CSR form)
        void *xp = nullptr;           // displacement copy, 6 per node (float or double)
        int32_t *pad_of_dof = nullptr;  // dof -> node * 6 + component
        bool ready = false;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int64_t graph_steps = 0;
        // external load g(t) Fmag: Fmag (n), g at the step indices (nmul), and
        // the step index of the current state on the device (advanced after
        // every batch of steps)
        double *Fmag = nullptr, *mul = nullptr;
        size_t cap_Fmag = 0, cap_mul = 0;
        int64_t nmul = 0;
        int64_t *step = nullptr;
        bool load = false;
    } ex;
    // tile shapes of the shell element kernel and of the gather (0: defaults)
    struct Tune {
        int mode = -1;         // -1: not read yet (FLEXSHELL_AUTOTUNE), 0 off, 1 on, 2 re-tune
        int elem_epb = 0;      // elements per block
        int gather_warps = 0;  // warps (nodes) per block
        int gather_once = -1;  // node-block pairs summed once: -1 default (yes), 0 no, 1 yes
        bool from_tuner = false;
    } tune;
    // batched meshes fused into one mesh (fs_batch_*): first matrix row of each
    struct Batch {
        bool active = false;
        std::vector<int64_t> roff;  // nmeshes + 1
    } batch;
    // co-rotational beams (FEMMCorotBeam)
    struct Beam {
        fs::BeamSection *sec = nullptr;  // per rank
        double E = 0, nu = 0, rho = 0;
        double *u1 = nullptr;            // 3 x nnodes (SoA)
        double *R1 = nullptr;            // 9 x nnodes (SoA), R[:] per node
        double *v1 = nullptr;            // 6 x nnodes (SoA)
        bool have_u = false, have_R = false, have_v = false;
        double *q = nullptr;             // distributed load, 3 per rank
        double *fe = nullptr;            // element vectors, 12 per rank
        double *F = nullptr;             // assembled vector
        size_t F_cap = 0;
        bool ready = false;
    } beam;
};

namespace fs {

// launchers (defined in the .cu files)
int launch_prepare_mesh(fs_ctx *c, const int64_t *d_conn_raw, const int64_t *d_order_raw,
                        const int64_t *d_dof_raw);
int launch_prepare_dofs(fs_ctx *c, const int64_t *d_dof_raw);
int build_adjacency(fs_ctx *c);
int build_pattern(fs_ctx *c, int64_t n);
int launch_normals(fs_ctx *c, int kind = FS_CSYS_ISOPARAMETRIC, const double *prm = nullptr);
int round_normals(fs_ctx *c);
int launch_elements(fs_ctx *c, int precision);
int launch_gather(fs_ctx *c, int precision, double *vals);
int launch_elements_to(fs_ctx *c, int precision, void *ke);
int launch_gather_from(fs_ctx *c, int precision, const void *ke, double *vals);
int launch_masses(fs_ctx *c);
int assemble_mass(fs_ctx *c, int assembler, int64_t n);
int compact_zeros(fs_ctx *c, int64_t n, const int64_t *rowptr, const int32_t *colidx,
                  const double *vals, int64_t nnz);
int exclusive_scan_i64(fs_ctx *c, const int64_t *in, int64_t *out, int64_t n, int64_t *total);
int ensure_scratch(fs_ctx *c, size_t bytes);
int read_status(fs_ctx *c, int *bits);
// FS_OK when the context holds a shell mesh with parameters (and, with
// need_dofs, a dof numbering) and its layups if layered; else the error code
int check_ready(fs_ctx *c, bool need_dofs = true);
// the error code and message of a kernel status word (DEV_* bits)
int status_to_code(fs_ctx *c, int bits);
// FS_OK when the context's current matrix is a stiffness (the last matrix
// assembled came from fs_stiffness or fs_beam_matrix with FS_BEAM_STIFFNESS),
// else FS_ERR_STATE: the entry points that use "the last stiffness"
int check_last_stiffness(fs_ctx *c);
// address of the allocation-free path's scratch array in the current CUDA
// context, looked up when the context is created (fs_noalloc.cu)
void noalloc_setup(fs_ctx *c);
// releases the shift-invert factor of the context (fs_eigen.cu)
void free_shift(fs_ctx *c);
// ends the explicit step's state and releases its captured steps, which read
// the pattern's neighbour lists and, in the CSR form, the current matrix:
// called before either changes (fs_explicit.cu)
void end_explicit(fs_ctx *c);

int explicit_launch_steps(fs_ctx *c, int64_t nsteps);

// tile-shape autotuner of the shell assembly
int autotune_shell(fs_ctx *c, int precision);
size_t t3_smem(int precision, bool avgk, bool layered, int epb);
size_t entry_bytes(int precision);
size_t gather_smem_bytes(int precision, int nen, int warps);
int run_t3_any(fs_ctx *c, int precision, void *ke);
int run_q4_any(fs_ctx *c, int precision, void *ke);
size_t q4_smem(int precision, bool layered, int epb);

// co-rotational beams
int launch_beam_elements(fs_ctx *c, int which, int mass_type);
int launch_beam_vector(fs_ctx *c, int which, int64_t n, double *F);
// per-node sums (ascending assembly rank) of element vectors fe (6 nen per rank) into F[0, n)
int launch_vec_gather(fs_ctx *c, int64_t n, const double *fe, double *F);
void free_beam(fs_ctx *c);
// pattern + element kernel + gather + assembler post-processing shared by the
// shells (beam_which < 0) and the beams
int assemble_matrix(fs_ctx *c, int precision, int assembler, int64_t nrows, int64_t *nnz_out, int beam_which,
                    int mass_type);

// helpers
int set_err(fs_ctx *c, int code, const std::string &msg);
int cuda_check(fs_ctx *c, cudaError_t e, const char *what);
template <class T> int dalloc(fs_ctx *c, T **p, size_t n)
{
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(c, FS_ERR_OOM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    return FS_OK;
}
template <class T> void dfree(T **p)
{
    if (*p) cudaFree(*p);
    *p = nullptr;
}
// device buffer of at least n elements, reused when its capacity suffices
template <class T> int grow(fs_ctx *c, T **p, size_t *cap, size_t n)
{
    if (*p && *cap >= n && n > 0) return FS_OK;
    const int st = dalloc(c, p, n);
    *cap = st == FS_OK ? (n ? n : 1) : 0;
    return st;
}

}  // namespace fs

#define FS_TRY(x)                 \
    do {                          \
        int _s = (x);             \
        if (_s != FS_OK) return _s; \
    } while (0)
#define FS_CUDA(c, call) FS_TRY(fs::cuda_check((c), (call), #call))

namespace fs {

// per-element host array (mesh order) -> device array by assembly rank
template <class T>
__global__ void k_by_rank(int64_t nelem, const int32_t *elem_of_rank, const T *src, T *dst)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nelem) dst[r] = src[elem_of_rank[r]];
}

template <class T>
int upload_by_rank(fs_ctx *c, const T *host, int64_t nelem, T **dst)
{
    FS_TRY(dalloc(c, dst, (size_t)nelem));
    if (nelem == 0) return FS_OK;
    T *tmp = nullptr;
    FS_TRY(dalloc(c, &tmp, (size_t)nelem));
    FS_CUDA(c, cudaMemcpyAsync(tmp, host, sizeof(T) * nelem, cudaMemcpyHostToDevice, c->stream));
    k_by_rank<T><<<(unsigned)((nelem + 255) / 256), 256, 0, c->stream>>>(nelem, c->mesh.elem_of_rank, tmp, *dst);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(tmp);
    return FS_OK;
}

}  // namespace fs

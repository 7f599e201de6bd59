// Co-rotational beams (FEMMCorotBeam, src/FEMMCorotBeamModule.jl): element
// kernels for the stiffness, geometric stiffness, mass and gyroscopic
// matrices, the restoring-force and distributed-load vectors, and the
// deterministic vector gather.
//
// One thread owns one element.  Matrices are stored like the shell element
// matrices: the upper 6x6 node blocks (3 per beam), row-major inside a
// block, by assembly rank; the shell gather (NEN = 2) turns them into CSR
// values.  Vectors are 12 doubles per rank; a node's six entries are summed
// over its (element, local node) pairs in ascending rank, so the result is
// the element-order sum of SysvecAssembler, bit-reproducible and without
// atomics.
#include <cmath>
#include <cstring>

#include "fs_internal.cuh"

static_assert(sizeof(fs_beam_section) == sizeof(fs::BeamSection), "section layouts differ");

namespace fs {

static unsigned nblk_b(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

struct V3 {
    double v[3];
};
static_assert(sizeof(V3) == 24, "V3");

struct BeamDev {
    const BeamSection *sec;
    const double *u1, *R1, *v1, *q;  // q: distributed load, 3 per rank
    double E, G, rho;
};

__device__ __forceinline__ void beam_load(const MeshDev &m, const BeamDev &b, int64_t r, double x0[2][3],
                                          double xt[2][3], double R[2][3][3])
{
    for (int a = 0; a < 2; a++) {
        const int node = m.conn[r * 2 + a];
        for (int c = 0; c < 3; c++) {
            x0[a][c] = m.xyz[(int64_t)c * m.nnodes + node];
            xt[a][c] = x0[a][c] + (b.u1 ? b.u1[(int64_t)c * m.nnodes + node] : 0.0);
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                R[a][i][j] = b.R1 ? b.R1[(int64_t)(i + 3 * j) * m.nnodes + node] : (i == j ? 1.0 : 0.0);
    }
}

__device__ __forceinline__ void store_block_d(double *o, const double (&acc)[6][6])
{
    double2 *o2 = reinterpret_cast<double2 *>(o);
#pragma unroll
    for (int q = 0; q < 18; q++) o2[q] = make_double2(acc[(2 * q) / 6][(2 * q) % 6], acc[(2 * q + 1) / 6][(2 * q + 1) % 6]);
}

__device__ __forceinline__ void beam_prepare_rank(const MeshDev &m, const BeamDev &b, int64_t r, bool velocities,
                                                  int mass_type, BeamElem &e)
{
    double x0[2][3], xt[2][3], R[2][3][3], v[2][6];
    beam_load(m, b, r, x0, xt, R);
    if (velocities)
        for (int a = 0; a < 2; a++) {
            const int node = m.conn[r * 2 + a];
            for (int k = 0; k < 6; k++) v[a][k] = b.v1 ? b.v1[(int64_t)k * m.nnodes + node] : 0.0;
        }
    beam_prepare(x0, xt, R, velocities ? v : nullptr, b.sec[r], b.E, b.G, b.rho, mass_type, e);
}

// upper node blocks (0,0), (0,1), (1,1) of element matrix WHICH
template <int WHICH>
__global__ void __launch_bounds__(128) k_beam_elements(const MeshDev m, const BeamDev b, int mass_type, double *ke)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nelem) return;
    BeamElem e;
    beam_prepare_rank(m, b, r, WHICH == FS_BEAM_GYROSCOPIC, mass_type, e);
    double *out = ke + r * 108;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int bb = a; bb < 2; bb++) {
            double acc[6][6];
            beam_block<WHICH>(e, a, bb, acc);
            store_block_d(out + ub(a, bb, 2) * 36, acc);
        }
}

// restoring force (WHICH 4) and distributed load (WHICH 5) per element
template <int WHICH>
__global__ void __launch_bounds__(128) k_beam_vectors(const MeshDev m, const BeamDev b, double *fe)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nelem) return;
    BeamElem e;
    beam_prepare_rank(m, b, r, false, 0, e);
    double out[12];
    if (WHICH == 4)
        beam_restoring(e, out);
    else
        beam_distribload(e, b.q + r * 3, out);
    double2 *o2 = reinterpret_cast<double2 *>(fe + r * 12);
#pragma unroll
    for (int q = 0; q < 6; q++) o2[q] = make_double2(out[2 * q], out[2 * q + 1]);
}

// node sums of element vectors in ascending assembly rank
__global__ void k_vec_gather(const MeshDev m, int64_t n, const double *fe, double *F)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nnodes) return;
    const int nd = 6 * m.nen;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t p = m.pp[r]; p < m.pp[r + 1]; p++) {
        const int32_t v = m.pair_e[p];
        const double *src = fe + (int64_t)(v >> 2) * nd + 6 * (v & 3);
#pragma unroll
        for (int k = 0; k < 6; k++) acc[k] += src[k];
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const int32_t d = m.dof[(int64_t)k * m.nnodes + r];
        if (d >= 1 && d <= n) F[d - 1] = acc[k];
    }
}

int launch_vec_gather(fs_ctx *c, int64_t n, const double *fe, double *F)
{
    const MeshDev &m = c->mesh;
    if (m.nnodes) k_vec_gather<<<nblk_b(m.nnodes, 128), 128, 0, c->stream>>>(m, n, fe, F);
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

static BeamDev beam_dev(fs_ctx *c)
{
    BeamDev b;
    b.sec = c->beam.sec;
    b.u1 = c->beam.have_u ? c->beam.u1 : nullptr;
    b.R1 = c->beam.have_R ? c->beam.R1 : nullptr;
    b.v1 = c->beam.have_v ? c->beam.v1 : nullptr;
    b.q = c->beam.q;
    b.E = c->beam.E;
    b.G = c->beam.E / 2 / (1 + c->beam.nu);
    b.rho = c->beam.rho;
    return b;
}

int launch_beam_elements(fs_ctx *c, int which, int mass_type)
{
    MeshDev &m = c->mesh;
    const size_t bytes = (size_t)m.nelem * 108 * sizeof(double);
    if (bytes > c->ke_bytes || !c->ke) {
        if (c->ke) cudaFree(c->ke);
        c->ke = nullptr;
        c->ke_bytes = 0;
        cudaError_t e = cudaMalloc(&c->ke, bytes ? bytes : 16);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_err(c, FS_ERR_OOM, "device allocation of element matrices failed");
        }
        c->ke_bytes = bytes;
    }
    if (m.nelem == 0) return FS_OK;
    const BeamDev b = beam_dev(c);
    double *ke = (double *)c->ke;
    const unsigned g = nblk_b(m.nelem, 128);
    switch (which) {
    case FS_BEAM_STIFFNESS: k_beam_elements<FS_BEAM_STIFFNESS><<<g, 128, 0, c->stream>>>(m, b, mass_type, ke); break;
    case FS_BEAM_GEOSTIFFNESS: k_beam_elements<FS_BEAM_GEOSTIFFNESS><<<g, 128, 0, c->stream>>>(m, b, mass_type, ke); break;
    case FS_BEAM_MASS: k_beam_elements<FS_BEAM_MASS><<<g, 128, 0, c->stream>>>(m, b, mass_type, ke); break;
    default: k_beam_elements<FS_BEAM_GYROSCOPIC><<<g, 128, 0, c->stream>>>(m, b, mass_type, ke); break;
    }
    FS_CUDA(c, cudaGetLastError());
    return FS_OK;
}

// element vectors into c->beam.fe; assembled into F (device, n entries) when F is given
int launch_beam_vector(fs_ctx *c, int which, int64_t n, double *F)
{
    MeshDev &m = c->mesh;
    FS_TRY(dalloc(c, &c->beam.fe, (size_t)(12 * m.nelem)));
    const BeamDev b = beam_dev(c);
    if (m.nelem) {
        const unsigned g = nblk_b(m.nelem, 128);
        if (which == 4)
            k_beam_vectors<4><<<g, 128, 0, c->stream>>>(m, b, c->beam.fe);
        else
            k_beam_vectors<5><<<g, 128, 0, c->stream>>>(m, b, c->beam.fe);
        FS_CUDA(c, cudaGetLastError());
    }
    if (F) {
        if (n > 0) FS_CUDA(c, cudaMemsetAsync(F, 0, sizeof(double) * n, c->stream));
        FS_TRY(launch_vec_gather(c, n, c->beam.fe, F));
    }
    return FS_OK;
}

void free_beam(fs_ctx *c)
{
    dfree(&c->beam.sec);
    dfree(&c->beam.u1);
    dfree(&c->beam.R1);
    dfree(&c->beam.v1);
    dfree(&c->beam.q);
    dfree(&c->beam.fe);
    dfree(&c->beam.F);
    c->beam = fs_ctx::Beam();
}

static int beam_check(fs_ctx *c)
{
    if (c->mesh.etype != FS_COROTBEAM) return set_err(c, FS_ERR_STATE, "no beam mesh: call fs_mesh_set with FS_COROTBEAM");
    if (!c->beam.ready) return set_err(c, FS_ERR_STATE, "no cross sections: call fs_beam_setup first");
    return FS_OK;
}

// distributed load per rank from the caller's array (one 3-vector, or one per element in mesh order)
static int upload_load(fs_ctx *c, const double *q, int per_element)
{
    MeshDev &m = c->mesh;
    if (!q) return set_err(c, FS_ERR_BAD_INPUT, "missing load array");
    std::vector<double> h((size_t)(3 * m.nelem));
    for (int64_t e = 0; e < m.nelem; e++)
        for (int k = 0; k < 3; k++) h[(size_t)(3 * e + k)] = per_element ? q[3 * e + k] : q[k];
    // to rank order: upload as 3-vectors by rank
    V3 *dq = nullptr;
    FS_TRY(upload_by_rank<V3>(c, reinterpret_cast<const V3 *>(h.data()), m.nelem, &dq));
    dfree(&c->beam.q);
    c->beam.q = reinterpret_cast<double *>(dq);
    return FS_OK;
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_beam_setup(fs_ctx *c, const fs_beam_section *sections, double E, double nu, double rho)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype != FS_COROTBEAM) return set_err(c, FS_ERR_STATE, "no beam mesh: call fs_mesh_set with FS_COROTBEAM");
    if (c->mesh.nelem && !sections) return set_err(c, FS_ERR_BAD_INPUT, "missing sections");
    if (!(E > 0.0) || !(nu > -1.0 && nu < 0.5) || !(rho >= 0.0))
        return set_err(c, FS_ERR_BAD_INPUT, "material constants out of range (E > 0, -1 < nu < 0.5, rho >= 0)");
    for (int64_t e = 0; e < c->mesh.nelem; e++) {
        const fs_beam_section &s = sections[e];
        if (!(s.A > 0.0) || !(s.J >= 0.0) || !(s.I1 >= 0.0) || !(s.I2 >= 0.0) || !(s.I3 >= 0.0) || !(s.A2s > 0.0) ||
            !(s.A3s > 0.0))
            return set_err(c, FS_ERR_BAD_INPUT, "cross section with a non-positive area or negative moment");
    }
    FS_TRY(upload_by_rank<BeamSection>(c, reinterpret_cast<const BeamSection *>(sections), c->mesh.nelem,
                                       &c->beam.sec));
    c->beam.E = E;
    c->beam.nu = nu;
    c->beam.rho = rho;
    c->beam.ready = true;
    return FS_OK;
}

int fs_beam_state_set(fs_ctx *c, const double *u1, const double *R1, const double *v1)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (c->mesh.etype != FS_COROTBEAM) return set_err(c, FS_ERR_STATE, "no beam mesh: call fs_mesh_set with FS_COROTBEAM");
    const int64_t nn = c->mesh.nnodes;
    struct In { const double *h; double **d; bool *have; int w; } ins[3] = {
        {u1, &c->beam.u1, &c->beam.have_u, 3}, {R1, &c->beam.R1, &c->beam.have_R, 9}, {v1, &c->beam.v1, &c->beam.have_v, 6}};
    for (auto &x : ins) {
        *x.have = x.h != nullptr;
        if (!x.h || nn == 0) continue;
        if (!*x.d) FS_TRY(dalloc(c, x.d, (size_t)(x.w * nn)));
        FS_CUDA(c, cudaMemcpyAsync(*x.d, x.h, sizeof(double) * x.w * nn, cudaMemcpyHostToDevice, c->stream));
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_beam_matrix(fs_ctx *c, int which, int mass_type, int assembler, int64_t nrows, int64_t *nnz_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(beam_check(c));
    if (!c->dofs_ready) return set_err(c, FS_ERR_STATE, "no dof numbering: call fs_dofs_set first");
    if (which < FS_BEAM_STIFFNESS || which > FS_BEAM_GYROSCOPIC) return set_err(c, FS_ERR_BAD_INPUT, "unknown beam matrix");
    if (mass_type < 0 || mass_type > 3) return set_err(c, FS_ERR_BAD_INPUT, "unknown mass_type");
    if (assembler < FS_ASM_SPARSE || assembler > FS_ASM_DIAG) return set_err(c, FS_ERR_BAD_INPUT, "unknown assembler");
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative matrix size");
    return assemble_matrix(c, FS_FP64, assembler, nrows, nnz_out, which, mass_type);
}

static int beam_vector_out(fs_ctx *c, int which, int64_t nrows, double *F)
{
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative vector size");
    if (nrows && !F) return set_err(c, FS_ERR_BAD_INPUT, "missing output vector");
    if (!c->dofs_ready) return set_err(c, FS_ERR_STATE, "no dof numbering: call fs_dofs_set first");
    if ((size_t)nrows > c->beam.F_cap || !c->beam.F) {
        FS_TRY(dalloc(c, &c->beam.F, (size_t)nrows));
        c->beam.F_cap = (size_t)nrows;
    }
    FS_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    FS_TRY(launch_beam_vector(c, which, nrows, c->beam.F));
    FS_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    if (nrows) FS_CUDA(c, cudaMemcpyAsync(F, c->beam.F, sizeof(double) * nrows, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_beam_restoringforce(fs_ctx *c, int64_t nrows, double *F)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(beam_check(c));
    return beam_vector_out(c, 4, nrows, F);
}

int fs_beam_distribloads_global(fs_ctx *c, const double *q, int per_element, int64_t nrows, double *F)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(beam_check(c));
    FS_TRY(upload_load(c, q, per_element));
    return beam_vector_out(c, 5, nrows, F);
}

int fs_beam_element_matrices(fs_ctx *c, int which, int mass_type, double *out)
{
    if (!c || !out) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(beam_check(c));
    if (which < FS_BEAM_STIFFNESS || which > FS_BEAM_GYROSCOPIC) return set_err(c, FS_ERR_BAD_INPUT, "unknown beam matrix");
    if (mass_type < 0 || mass_type > 3) return set_err(c, FS_ERR_BAD_INPUT, "unknown mass_type");
    FS_TRY(launch_beam_elements(c, which, mass_type));
    const int64_t ne = c->mesh.nelem;
    std::vector<double> blk((size_t)(108 * ne));
    std::vector<int32_t> eor((size_t)ne);
    if (ne) {
        FS_CUDA(c, cudaMemcpyAsync(blk.data(), c->ke, sizeof(double) * 108 * ne, cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaMemcpyAsync(eor.data(), c->mesh.elem_of_rank, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost,
                                   c->stream));
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int64_t r = 0; r < ne; r++) {
        double *o = out + (int64_t)144 * eor[(size_t)r];
        const double *k = blk.data() + 108 * r;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++)
                        o[(6 * a + i) + 12 * (6 * b + j)] =
                            a <= b ? k[ub(a, b, 2) * 36 + i * 6 + j] : k[ub(b, a, 2) * 36 + j * 6 + i];
    }
    return FS_OK;
}

int fs_beam_element_vectors(fs_ctx *c, int which, const double *q, int per_element, double *out)
{
    if (!c || !out) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(beam_check(c));
    if (which != 4 && which != 5) return set_err(c, FS_ERR_BAD_INPUT, "unknown beam vector (4 restoring force, 5 load)");
    if (which == 5) FS_TRY(upload_load(c, q, per_element));
    FS_TRY(launch_beam_vector(c, which, 0, nullptr));
    const int64_t ne = c->mesh.nelem;
    std::vector<double> v((size_t)(12 * ne));
    std::vector<int32_t> eor((size_t)ne);
    if (ne) {
        FS_CUDA(c, cudaMemcpyAsync(v.data(), c->beam.fe, sizeof(double) * 12 * ne, cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaMemcpyAsync(eor.data(), c->mesh.elem_of_rank, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost,
                                   c->stream));
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int64_t r = 0; r < ne; r++) memcpy(out + 12 * (int64_t)eor[(size_t)r], v.data() + 12 * r, sizeof(double) * 12);
    return FS_OK;
}

}  // extern "C"

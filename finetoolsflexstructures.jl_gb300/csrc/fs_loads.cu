// Distributed loads on the shell meshes and their boundary curves:
// distribloads(FEMMBase(IntegDomain(fes, rule)), geom0, dchi, fi, m) of
// FinEtools 8.2.5 (FEMMBaseModule), as the reference calls it on its shell
// element sets (examples/shells/dynamics/homogeneous/explicit/
// plate_expl_examples.jl:196-199, test/test_shell_statics.jl:84-86,
// test/test_shell_resultants.jl:108-110) and on the two-node line elements of
// a shell mesh's boundary (meshboundary, GaussRule(1, 2):
// test/test_shell_statics.jl:212-215, test/test_composite_shell_statics.jl:
// 80-88).  Per element and integration point the load intensity f (six
// components, one per nodal dof) contributes N_a(xi) J(xi) w f to node a, J
// the surface Jacobian |x,xi x x,eta| or, on a line element, the curve
// Jacobian |x,xi| (times the other dimension 1 for the higher manifold
// dimensions m, as FEMMBase's default); the element vectors
// are summed per node in ascending assembly rank, the element-order sum of
// FinEtools' vector assembler.  One thread per element, double precision.
#include "fs_internal.cuh"

namespace fs {

// integration points on the parent element; T3: TriRule(npts), npts 1, 3 or 6
// (the centroid; the degree-2 interior rule; Dunavant's degree-4 rule),
// weights summing to 1/2; Q4: GaussRule(2, order), order 1, 2 or 3, tensor
// points with xi the outer index, weights summing to 4; L2: GaussRule(1,
// order), order 1, 2 or 3, weights summing to 2 (eta unused)
struct SurfRule {
    int npts = 0;
    double xi[9], eta[9], w[9];
};

static bool make_rule(int nen, int rule, SurfRule &R)
{
    if (nen == 3) {
        if (rule == 1) {
            R.npts = 1;
            R.xi[0] = R.eta[0] = 1.0 / 3.0;
            R.w[0] = 0.5;
        } else if (rule == 3) {
            const double a = 2.0 / 3.0, b = 1.0 / 6.0;
            const double xi[3] = {a, b, b}, eta[3] = {b, a, b};
            R.npts = 3;
            for (int j = 0; j < 3; j++) {
                R.xi[j] = xi[j];
                R.eta[j] = eta[j];
                R.w[j] = 1.0 / 6.0;
            }
        } else if (rule == 6) {
            // D. A. Dunavant, High degree efficient symmetrical Gaussian
            // quadrature rules for the triangle (1985), degree 4: two orbits
            // of three points (barycentric (1 - 2a, a, a) and permutations)
            const double a1 = 0.445948490915965, w1 = 0.223381589678011;
            const double a2 = 0.091576213509771, w2 = 0.109951743655322;
            const double A[2] = {a1, a2}, W[2] = {w1, w2};
            R.npts = 6;
            for (int o = 0; o < 2; o++) {
                const double a = A[o], c = 1.0 - 2.0 * a;
                const double xi[3] = {c, a, a}, eta[3] = {a, c, a};
                for (int j = 0; j < 3; j++) {
                    R.xi[3 * o + j] = xi[j];
                    R.eta[3 * o + j] = eta[j];
                    R.w[3 * o + j] = W[o] / 2.0;
                }
            }
        } else {
            return false;
        }
        return true;
    }
    if (rule < 1 || rule > 3) return false;
    double pc[3], pw[3];
    if (rule == 1) {
        pc[0] = 0.0;
        pw[0] = 2.0;
    } else if (rule == 2) {
        pc[0] = -1.0 / sqrt(3.0);
        pc[1] = 1.0 / sqrt(3.0);
        pw[0] = pw[1] = 1.0;
    } else {
        pc[0] = -sqrt(0.6);
        pc[1] = 0.0;
        pc[2] = sqrt(0.6);
        pw[0] = pw[2] = 5.0 / 9.0;
        pw[1] = 8.0 / 9.0;
    }
    if (nen == 2) {
        R.npts = rule;
        for (int i = 0; i < rule; i++) {
            R.xi[i] = pc[i];
            R.eta[i] = 0.0;
            R.w[i] = pw[i];
        }
        return true;
    }
    R.npts = rule * rule;
    for (int i = 0; i < rule; i++)
        for (int j = 0; j < rule; j++) {
            R.xi[i * rule + j] = pc[i];
            R.eta[i * rule + j] = pc[j];
            R.w[i * rule + j] = pw[i] * pw[j];
        }
    return true;
}

// shape functions and their parent derivatives at (xi, eta)
template <int NN>
__device__ __forceinline__ void surf_basis(double xi, double eta, double N[NN], double dx[NN], double de[NN])
{
    if constexpr (NN == 2) {
        N[0] = 0.5 * (1.0 - xi);
        N[1] = 0.5 * (1.0 + xi);
        dx[0] = -0.5; dx[1] = 0.5;
        de[0] = 0.0; de[1] = 0.0;
    } else if constexpr (NN == 3) {
        N[0] = 1.0 - xi - eta;
        N[1] = xi;
        N[2] = eta;
        dx[0] = -1.0; dx[1] = 1.0; dx[2] = 0.0;
        de[0] = -1.0; de[1] = 0.0; de[2] = 1.0;
    } else {
        const double xm = 1.0 - xi, xp = 1.0 + xi, em = 1.0 - eta, ep = 1.0 + eta;
        N[0] = 0.25 * xm * em;
        N[1] = 0.25 * xp * em;
        N[2] = 0.25 * xp * ep;
        N[3] = 0.25 * xm * ep;
        dx[0] = -0.25 * em; dx[1] = 0.25 * em; dx[2] = 0.25 * ep; dx[3] = -0.25 * ep;
        de[0] = -0.25 * xm; de[1] = -0.25 * xp; de[2] = 0.25 * xp; de[3] = 0.25 * xm;
    }
}

// location, tangents and surface Jacobian of point j of the element of rank r
template <int NN>
__device__ __forceinline__ void surf_point(const MeshDev &m, const SurfRule &R, int64_t r, int j, double N[NN],
                                           double loc[3], double t1[3], double t2[3])
{
    double dx[NN], de[NN];
    surf_basis<NN>(R.xi[j], R.eta[j], N, dx, de);
    for (int i = 0; i < 3; i++) loc[i] = t1[i] = t2[i] = 0.0;
    for (int a = 0; a < NN; a++) {
        const int64_t node = m.conn[r * NN + a];
        for (int i = 0; i < 3; i++) {
            const double x = m.xyz[(int64_t)i * m.nnodes + node];
            loc[i] += N[a] * x;
            t1[i] += x * dx[a];
            t2[i] += x * de[a];
        }
    }
}

template <int NN>
__global__ void __launch_bounds__(128) k_surface_loads(const MeshDev m, const SurfRule R, const double *f,
                                                       int64_t nf, double *fe)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m.nelem) return;
    const int64_t q = m.elem_of_rank[r];
    double F[6 * NN];
    for (int k = 0; k < 6 * NN; k++) F[k] = 0.0;
    for (int j = 0; j < R.npts; j++) {
        double N[NN], loc[3], t1[3], t2[3];
        surf_point<NN>(m, R, r, j, N, loc, t1, t2);
        double jac;
        if constexpr (NN == 2) {
            jac = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        } else {
            const double c1 = t1[1] * t2[2] - t1[2] * t2[1];
            const double c2 = t1[2] * t2[0] - t1[0] * t2[2];
            const double c3 = t1[0] * t2[1] - t1[1] * t2[0];
            jac = sqrt(c1 * c1 + c2 * c2 + c3 * c3);
        }
        const double factor = jac * R.w[j];
        const double *fp = nf == 1 ? f : (nf == m.nelem ? f + 6 * q : f + 6 * (q * R.npts + j));
        for (int a = 0; a < NN; a++) {
            const double nf_a = N[a] * factor;
            for (int k = 0; k < 6; k++) F[6 * a + k] += nf_a * fp[k];
        }
    }
    double2 *o2 = reinterpret_cast<double2 *>(fe + r * 6 * NN);
#pragma unroll
    for (int k = 0; k < 3 * NN; k++) o2[k] = make_double2(F[2 * k], F[2 * k + 1]);
}

// point data in element order: location, then the two parent tangents (the
// second zero on a line element)
template <int NN>
__global__ void __launch_bounds__(128) k_surface_points(const MeshDev m, const SurfRule R, double *out)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m.nelem * R.npts) return;
    const int64_t r = p / R.npts;
    const int j = (int)(p - r * R.npts);
    double N[NN], loc[3], t1[3], t2[3];
    surf_point<NN>(m, R, r, j, N, loc, t1, t2);
    double *o = out + 9 * ((int64_t)m.elem_of_rank[r] * R.npts + j);
    for (int i = 0; i < 3; i++) {
        o[i] = loc[i];
        o[3 + i] = t1[i];
        o[6 + i] = t2[i];
    }
}

static int check_surface(fs_ctx *c, int rule, SurfRule &R)
{
    const MeshDev &m = c->mesh;
    if (m.etype < 0) return set_err(c, FS_ERR_STATE, "no mesh: call fs_mesh_set first");
    // a two-node mesh (FS_COROTBEAM) is the L2 element set of the load
    if (!make_rule(m.nen, rule, R))
        return set_err(c, FS_ERR_BAD_INPUT,
                       m.nen == 3 ? "triangle rule: TriRule npts 1, 3 or 6"
                                  : (m.nen == 2 ? "line rule: GaussRule(1, order), order 1, 2 or 3"
                                                : "quadrilateral rule: GaussRule(2, order), order 1, 2 or 3"));
    return FS_OK;
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_integration_points(fs_ctx *c, int rule, double *out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    SurfRule R;
    FS_TRY(check_surface(c, rule, R));
    const MeshDev &m = c->mesh;
    const int64_t np = m.nelem * R.npts;
    if (np == 0) return FS_OK;
    if (!out) return set_err(c, FS_ERR_BAD_INPUT, "missing array");
    FS_TRY(ensure_scratch(c, sizeof(double) * 9 * (size_t)np));
    double *d = (double *)c->scratch;
    const unsigned g = (unsigned)((np + 127) / 128);
    if (m.nen == 2)
        k_surface_points<2><<<g, 128, 0, c->stream>>>(m, R, d);
    else if (m.nen == 3)
        k_surface_points<3><<<g, 128, 0, c->stream>>>(m, R, d);
    else
        k_surface_points<4><<<g, 128, 0, c->stream>>>(m, R, d);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaMemcpyAsync(out, d, sizeof(double) * 9 * np, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

int fs_distribloads(fs_ctx *c, int rule, int m_dim, const double *force, int64_t nforce, int64_t nrows, double *F)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    SurfRule R;
    FS_TRY(check_surface(c, rule, R));
    const MeshDev &m = c->mesh;
    if (m_dim < (m.nen == 2 ? 1 : 2) || m_dim > 3)
        return set_err(c, FS_ERR_BAD_INPUT, m.nen == 2 ? "m: 1 (curve), 2 or 3 (curve times the other dimension 1)"
                                                       : "m: 2 (surface) or 3 (surface times the other dimension 1)");
    if (!c->dofs_ready) return set_err(c, FS_ERR_STATE, "no dof numbering: call fs_dofs_set first");
    if (nrows < 0) return set_err(c, FS_ERR_BAD_INPUT, "negative vector length");
    const int64_t np = m.nelem * R.npts;
    if (nforce != 1 && nforce != m.nelem && nforce != np)
        return set_err(c, FS_ERR_BAD_INPUT, "force: one 6-vector, one per element or one per integration point");
    if ((nrows && !F) || !force) return set_err(c, FS_ERR_BAD_INPUT, "missing array");
    const size_t nfe = (size_t)(6 * m.nen) * (size_t)m.nelem, nfv = 6 * (size_t)nforce;
    FS_TRY(ensure_scratch(c, sizeof(double) * (nfe + nfv + (size_t)nrows) + 16));
    double *dfe = (double *)c->scratch, *df = dfe + nfe, *dF = df + nfv;
    FS_CUDA(c, cudaMemcpyAsync(df, force, sizeof(double) * nfv, cudaMemcpyHostToDevice, c->stream));
    if (m.nelem) {
        const unsigned g = (unsigned)((m.nelem + 127) / 128);
        if (m.nen == 2)
            k_surface_loads<2><<<g, 128, 0, c->stream>>>(m, R, df, nforce, dfe);
        else if (m.nen == 3)
            k_surface_loads<3><<<g, 128, 0, c->stream>>>(m, R, df, nforce, dfe);
        else
            k_surface_loads<4><<<g, 128, 0, c->stream>>>(m, R, df, nforce, dfe);
        FS_CUDA(c, cudaGetLastError());
    }
    if (nrows) {
        FS_CUDA(c, cudaMemsetAsync(dF, 0, sizeof(double) * nrows, c->stream));
        FS_TRY(launch_vec_gather(c, nrows, dfe, dF));
        FS_CUDA(c, cudaMemcpyAsync(F, dF, sizeof(double) * nrows, cudaMemcpyDeviceToHost, c->stream));
    }
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // extern "C"

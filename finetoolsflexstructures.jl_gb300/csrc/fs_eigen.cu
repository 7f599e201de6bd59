// Shift-invert support for the lowest modes of (K, M): a banded Cholesky
// factor of K - sigma M on the device and solves with it (fs_shift_factor,
// fs_shift_solve), the inner step of the reference's eigs(K, M; nev,
// which = :SM) with a shift (ARPACK's shift-invert mode,
// test/test_shell_dynamics.jl:79-80, test/test_composite_shell_dynamics.jl).
//
// Storage.  The matrix is symmetric with half-bandwidth kd (the largest
// i - j of a stored entry under the dof numbering).  Its lower band is kept
// column by column with leading dimension ld = kd + 2 NB: entry (i, j),
// 0 <= i - j < ld, at ab[(i - j) + j ld] = ab[i + j (ld - 1)].  Read with
// leading dimension ld - 1 the array is therefore an ordinary column-major
// matrix, and every block the factorisation touches (the NB x NB diagonal
// block, the kd x NB panel below it, the kd x kd trailing triangle) is a
// dense sub-matrix of that view.  Rows kd+1 .. kd+NB-1 of a column hold the
// panel's entries beyond the band, which are zero and stay zero.  In the
// view, the strictly upper triangle of a diagonal w x w block (w <= NB) lies
// on rows ld-w+1 .. ld-1 of other columns: the last NB rows are kept free so
// that a library routine touching those entries changes nothing in use.
//
// Factorisation (right-looking, blocked, lower): for each block column k,
// potrf of the diagonal block, trsm of the panel below it, and the update
// of the trailing triangle column panel by column panel (syrk of each
// NB x NB diagonal block, gemm of the rectangle below it) -- cuSOLVER and
// cuBLAS dense routines on those views, in double (cuBLAS in its pedantic
// math mode: no reduced-precision or emulated arithmetic).  The strictly upper triangle of a diagonal block's view lies on
// the padding rows of the panel beside it, so the block is factorised in a
// separate NB x NB buffer and only its lower triangle is copied back.  Solves: block forward and backward substitution (trsv/gemv for
// one right-hand side, trsm/gemm for several).
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "fs_internal.cuh"

namespace fs {

// cuBLAS and cuSOLVER are opened on the first factorisation (dlopen), so the
// library itself loads without them and shares the copies already loaded in
// the process, if any.
struct DenseLibs {
    bool ok = false;
    std::string err;
    decltype(&cublasCreate_v2) create;
    decltype(&cublasDestroy_v2) destroy;
    decltype(&cublasSetStream_v2) set_stream;
    decltype(&cublasSetPointerMode_v2) set_pointer_mode;
    decltype(&cublasSetMathMode) set_math_mode;
    decltype(&cublasDtrsv_v2) trsv;
    decltype(&cublasDgemv_v2) gemv;
    decltype(&cublasDtrsm_v2) trsm;
    decltype(&cublasDgemm_v2) gemm;
    decltype(&cublasDsyrk_v2) syrk;
    decltype(&cusolverDnCreate) dn_create;
    decltype(&cusolverDnDestroy) dn_destroy;
    decltype(&cusolverDnSetStream) dn_set_stream;
    decltype(&cusolverDnDpotrf_bufferSize) potrf_buffer;
    decltype(&cusolverDnDpotrf) potrf;
};

static void *open_first(const char *const *names)
{
    for (int i = 0; names[i]; i++) {
        void *h = dlopen(names[i], RTLD_NOW | RTLD_GLOBAL);
        if (h) return h;
    }
    return nullptr;
}

template <class F> static bool sym(void *h, const char *name, F *out)
{
    *out = reinterpret_cast<F>(dlsym(h, name));
    return *out != nullptr;
}

static const DenseLibs &dense_libs()
{
    static DenseLibs L;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *blas_names[] = {"libcublas.so.13", "libcublas.so", nullptr};
        const char *solver_names[] = {"libcusolver.so.12", "libcusolver.so", nullptr};
        void *hb = open_first(blas_names);
        void *hs = hb ? open_first(solver_names) : nullptr;
        if (!hb || !hs) {
            const char *e = dlerror();
            L.err = std::string("cannot open ") + (hb ? "libcusolver" : "libcublas") + ": " + (e ? e : "");
            return;
        }
        bool ok = sym(hb, "cublasCreate_v2", &L.create) && sym(hb, "cublasDestroy_v2", &L.destroy) &&
                  sym(hb, "cublasSetStream_v2", &L.set_stream) &&
                  sym(hb, "cublasSetPointerMode_v2", &L.set_pointer_mode) &&
                  sym(hb, "cublasSetMathMode", &L.set_math_mode) && sym(hb, "cublasDtrsv_v2", &L.trsv) &&
                  sym(hb, "cublasDgemv_v2", &L.gemv) && sym(hb, "cublasDtrsm_v2", &L.trsm) &&
                  sym(hb, "cublasDgemm_v2", &L.gemm) && sym(hb, "cublasDsyrk_v2", &L.syrk) &&
                  sym(hs, "cusolverDnCreate", &L.dn_create) && sym(hs, "cusolverDnDestroy", &L.dn_destroy) &&
                  sym(hs, "cusolverDnSetStream", &L.dn_set_stream) &&
                  sym(hs, "cusolverDnDpotrf_bufferSize", &L.potrf_buffer) && sym(hs, "cusolverDnDpotrf", &L.potrf);
        if (!ok) {
            L.err = "cuBLAS / cuSOLVER entry point missing";
            return;
        }
        L.ok = true;
    });
    return L;
}

static const int64_t BAND_NB = 256;

struct ShiftFactor {
    int64_t n = 0, kd = 0, ld = 0;
    double sigma = 0.0;
    double *ab = nullptr;
    size_t ab_cap = 0;  // doubles
    double *work = nullptr;
    int lwork = 0;
    int *info = nullptr;  // one per block column
    size_t info_cap = 0;
    double *x = nullptr;
    size_t x_cap = 0;
    double *w11 = nullptr;  // the diagonal block being factorised (NB x NB)
    unsigned long long *d_kd = nullptr;
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t sol = nullptr;
    bool ready = false;
};

void free_shift(fs_ctx *c)
{
    ShiftFactor *s = (ShiftFactor *)c->shift;
    if (!s) return;
    dfree(&s->ab); dfree(&s->work); dfree(&s->info); dfree(&s->x); dfree(&s->d_kd); dfree(&s->w11);
    if (s->blas) dense_libs().destroy(s->blas);
    if (s->sol) dense_libs().dn_destroy(s->sol);
    delete s;
    c->shift = nullptr;
}

// half-bandwidth: the largest i - (first column of row i) over the rows
__global__ void k_row_band(int64_t n, const int64_t *rowptr, const int32_t *colidx, unsigned long long *kd)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (rowptr[i + 1] > rowptr[i]) {
        const int64_t d = i - (int64_t)colidx[rowptr[i]];
        if (d > 0) atomicMax(kd, (unsigned long long)d);
    }
}

// lower band of K - sigma diag(m): row i's entries j <= i into column j
__global__ void k_fill_band(int64_t n, const int64_t *rowptr, const int32_t *colidx, const double *vals,
                            double sigma, const double *mdiag, int64_t ld, double *ab)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t q = rowptr[i]; q < rowptr[i + 1]; q++) {
        const int64_t j = colidx[q];
        if (j > i) break;
        double v = vals[q];
        if (j == i) v -= sigma * mdiag[i];
        ab[(i - j) + j * ld] = v;
    }
}

// the lower triangle (with the diagonal) of an nb x nb block between two
// column-major layouts; the other triangle of dst is left as it is
__global__ void k_copy_lower(int nb, const double *src, int64_t lds, double *dst, int64_t ldd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < nb && i >= j) dst[i + j * ldd] = src[i + j * lds];
}

static int blas_check(fs_ctx *c, cublasStatus_t st, const char *what)
{
    if (st == CUBLAS_STATUS_SUCCESS) return FS_OK;
    return set_err(c, FS_ERR_CUDA, std::string(what) + " failed (cuBLAS status " + std::to_string((int)st) + ")");
}
static int solver_check(fs_ctx *c, cusolverStatus_t st, const char *what)
{
    if (st == CUSOLVER_STATUS_SUCCESS) return FS_OK;
    return set_err(c, FS_ERR_CUDA, std::string(what) + " failed (cuSOLVER status " + std::to_string((int)st) + ")");
}
#define FS_BLAS(c, call) FS_TRY(blas_check((c), (call), #call))
#define FS_SOLVER(c, call) FS_TRY(solver_check((c), (call), #call))

static int shift_handles(fs_ctx *c, ShiftFactor **out)
{
    const DenseLibs &D = dense_libs();
    if (!D.ok) return set_err(c, FS_ERR_UNSUPPORTED, "shift-invert factor needs cuBLAS and cuSOLVER: " + D.err);
    if (!c->shift) c->shift = new ShiftFactor();
    ShiftFactor *s = (ShiftFactor *)c->shift;
    if (!s->blas) {
        FS_BLAS(c, D.create(&s->blas));
        FS_BLAS(c, D.set_stream(s->blas, c->stream));
        FS_BLAS(c, D.set_pointer_mode(s->blas, CUBLAS_POINTER_MODE_HOST));
        FS_BLAS(c, D.set_math_mode(s->blas, CUBLAS_PEDANTIC_MATH));
    }
    if (!s->sol) {
        FS_SOLVER(c, D.dn_create(&s->sol));
        FS_SOLVER(c, D.dn_set_stream(s->sol, c->stream));
    }
    *out = s;
    return FS_OK;
}

// x (n x nrhs, leading dimension n, on the device) <- (L L^T)^{-1} x
static int band_solve(fs_ctx *c, ShiftFactor *s, int nrhs, double *x)
{
    const DenseLibs &D = dense_libs();
    const int64_t n = s->n, kd = s->kd, ld = s->ld, lda = ld - 1;
    const double one = 1.0, mone = -1.0;
    const int64_t nblk = (n + BAND_NB - 1) / BAND_NB;
    for (int64_t b = 0; b < nblk; b++) {
        const int64_t k = b * BAND_NB, nb = std::min(BAND_NB, n - k), m = std::min(kd, n - k - nb);
        const double *A11 = s->ab + k * ld, *A21 = s->ab + k * ld + nb;
        if (nrhs == 1) {
            FS_BLAS(c, D.trsv(s->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, (int)nb, A11,
                                   (int)lda, x + k, 1));
            if (m > 0)
                FS_BLAS(c, D.gemv(s->blas, CUBLAS_OP_N, (int)m, (int)nb, &mone, A21, (int)lda, x + k, 1, &one,
                                       x + k + nb, 1));
        } else {
            FS_BLAS(c, D.trsm(s->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)nb, nrhs, &one, A11, (int)lda, x + k, (int)n));
            if (m > 0)
                FS_BLAS(c, D.gemm(s->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, nrhs, (int)nb, &mone, A21, (int)lda,
                                       x + k, (int)n, &one, x + k + nb, (int)n));
        }
    }
    for (int64_t b = nblk - 1; b >= 0; b--) {
        const int64_t k = b * BAND_NB, nb = std::min(BAND_NB, n - k), m = std::min(kd, n - k - nb);
        const double *A11 = s->ab + k * ld, *A21 = s->ab + k * ld + nb;
        if (nrhs == 1) {
            if (m > 0)
                FS_BLAS(c, D.gemv(s->blas, CUBLAS_OP_T, (int)m, (int)nb, &mone, A21, (int)lda, x + k + nb, 1,
                                       &one, x + k, 1));
            FS_BLAS(c, D.trsv(s->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, (int)nb, A11,
                                   (int)lda, x + k, 1));
        } else {
            if (m > 0)
                FS_BLAS(c, D.gemm(s->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)nb, nrhs, (int)m, &mone, A21, (int)lda,
                                       x + k + nb, (int)n, &one, x + k, (int)n));
            FS_BLAS(c, D.trsm(s->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                                   CUBLAS_DIAG_NON_UNIT, (int)nb, nrhs, &one, A11, (int)lda, x + k, (int)n));
        }
    }
    return FS_OK;
}

}  // namespace fs

using namespace fs;

extern "C" {

int fs_shift_factor(fs_ctx *c, double sigma, const double *mdiag, int64_t *bandwidth_out)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    FS_TRY(check_last_stiffness(c));
    const int64_t n = c->mat_n;
    if (n > 0 && !mdiag) return set_err(c, FS_ERR_BAD_INPUT, "missing mass diagonal");
    ShiftFactor *s = nullptr;
    FS_TRY(shift_handles(c, &s));
    const DenseLibs &D = dense_libs();
    s->ready = false;
    s->n = n;
    s->sigma = sigma;
    if (n == 0) {
        s->ready = true;
        if (bandwidth_out) *bandwidth_out = 0;
        return FS_OK;
    }
    if (!s->d_kd) FS_TRY(dalloc(c, &s->d_kd, 1));
    FS_CUDA(c, cudaMemsetAsync(s->d_kd, 0, sizeof(unsigned long long), c->stream));
    k_row_band<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, s->d_kd);
    FS_CUDA(c, cudaGetLastError());
    unsigned long long kd = 0;
    FS_CUDA(c, cudaMemcpyAsync(&kd, s->d_kd, sizeof(kd), cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    s->kd = (int64_t)kd;
    s->ld = s->kd + 2 * BAND_NB;
    const double gib = (double)n * (double)s->ld * 8.0 / (1024.0 * 1024.0 * 1024.0);
    if (gib > 160.0) {
        char msg[240];
        snprintf(msg, sizeof(msg),
                 "band factor of %.1f GiB (half-bandwidth %lld for %lld rows) above the 160 GiB limit: number the "
                 "dofs for a smaller bandwidth (e.g. reverse Cuthill-McKee)",
                 gib, (long long)s->kd, (long long)n);
        return set_err(c, FS_ERR_UNSUPPORTED, msg);
    }
    FS_TRY(grow(c, &s->ab, &s->ab_cap, (size_t)(n * s->ld)));
    FS_CUDA(c, cudaMemsetAsync(s->ab, 0, sizeof(double) * (size_t)(n * s->ld), c->stream));
    double *dm = nullptr;
    FS_TRY(ensure_scratch(c, sizeof(double) * (size_t)n));
    dm = (double *)c->scratch;
    FS_CUDA(c, cudaMemcpyAsync(dm, mdiag, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    k_fill_band<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->mat_rowptr, c->mat_colidx, c->vals, sigma,
                                                                     dm, s->ld, s->ab);
    FS_CUDA(c, cudaGetLastError());
    const int64_t lda = s->ld - 1, nblk = (n + BAND_NB - 1) / BAND_NB;
    if (!s->w11) FS_TRY(dalloc(c, &s->w11, (size_t)(BAND_NB * BAND_NB)));
    FS_CUDA(c, cudaMemsetAsync(s->w11, 0, sizeof(double) * BAND_NB * BAND_NB, c->stream));
    int lw = 0;
    FS_SOLVER(c, D.potrf_buffer(s->sol, CUBLAS_FILL_MODE_LOWER, (int)BAND_NB, s->w11, (int)BAND_NB, &lw));
    if (lw > s->lwork || !s->work) {
        FS_TRY(dalloc(c, &s->work, (size_t)std::max(lw, 1)));
        s->lwork = std::max(lw, 1);
    }
    FS_TRY(grow(c, &s->info, &s->info_cap, (size_t)nblk));
    FS_CUDA(c, cudaMemsetAsync(s->info, 0, sizeof(int) * nblk, c->stream));
    const double one = 1.0, mone = -1.0;
    for (int64_t b = 0; b < nblk; b++) {
        const int64_t k = b * BAND_NB, nb = std::min(BAND_NB, n - k), m = std::min(s->kd, n - k - nb);
        double *A11 = s->ab + k * s->ld, *A21 = A11 + nb, *A22 = s->ab + (k + nb) * s->ld;
        const dim3 cg((unsigned)((nb + 127) / 128), (unsigned)nb);
        k_copy_lower<<<cg, 128, 0, c->stream>>>((int)nb, A11, lda, s->w11, BAND_NB);
        FS_CUDA(c, cudaGetLastError());
        FS_SOLVER(c, D.potrf(s->sol, CUBLAS_FILL_MODE_LOWER, (int)nb, s->w11, (int)BAND_NB, s->work, s->lwork,
                             s->info + b));
        k_copy_lower<<<cg, 128, 0, c->stream>>>((int)nb, s->w11, BAND_NB, A11, lda);
        FS_CUDA(c, cudaGetLastError());
        if (m > 0) {
            FS_BLAS(c, D.trsm(s->blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                                   CUBLAS_DIAG_NON_UNIT, (int)m, (int)nb, &one, s->w11, (int)BAND_NB, A21, (int)lda));
            for (int64_t p0 = 0; p0 < m; p0 += BAND_NB) {
                const int64_t w = std::min(BAND_NB, m - p0);
                FS_BLAS(c, D.syrk(s->blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, (int)w, (int)nb, &mone, A21 + p0,
                                  (int)lda, &one, A22 + p0 + p0 * lda, (int)lda));
                if (p0 + w < m)
                    FS_BLAS(c, D.gemm(s->blas, CUBLAS_OP_N, CUBLAS_OP_T, (int)(m - p0 - w), (int)w, (int)nb, &mone,
                                      A21 + p0 + w, (int)lda, A21 + p0, (int)lda, &one, A22 + p0 + w + p0 * lda,
                                      (int)lda));
            }
        }
    }
    std::vector<int> info((size_t)nblk);
    FS_CUDA(c, cudaMemcpyAsync(info.data(), s->info, sizeof(int) * nblk, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int64_t b = 0; b < nblk; b++)
        if (info[b] != 0) {
            char msg[200];
            snprintf(msg, sizeof(msg), "K - sigma M is not positive definite (leading minor %lld)",
                     (long long)(b * BAND_NB + info[b]));
            return set_err(c, FS_ERR_BAD_INPUT, msg);
        }
    s->ready = true;
    if (bandwidth_out) *bandwidth_out = s->kd;
    return FS_OK;
}

int fs_shift_solve(fs_ctx *c, int nrhs, const double *b, double *x)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    ShiftFactor *s = (ShiftFactor *)c->shift;
    if (!s || !s->ready) return set_err(c, FS_ERR_STATE, "no factor: call fs_shift_factor first");
    if (nrhs < 1) return set_err(c, FS_ERR_BAD_INPUT, "nrhs must be at least 1");
    const int64_t n = s->n;
    if (n == 0) return FS_OK;
    if (!b || !x) return set_err(c, FS_ERR_BAD_INPUT, "missing vector");
    const size_t len = (size_t)n * (size_t)nrhs;
    FS_TRY(grow(c, &s->x, &s->x_cap, len));
    FS_CUDA(c, cudaMemcpyAsync(s->x, b, sizeof(double) * len, cudaMemcpyHostToDevice, c->stream));
    FS_TRY(band_solve(c, s, nrhs, s->x));
    FS_CUDA(c, cudaMemcpyAsync(x, s->x, sizeof(double) * len, cudaMemcpyDeviceToHost, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

}  // extern "C"

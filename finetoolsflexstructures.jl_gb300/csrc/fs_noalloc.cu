// Allocation-free stiffness values (fs_stiffness_values_noalloc).
//
// Some callers cannot let the library allocate device memory when they ask
// for a stiffness: a host that hands the whole GPU to its own pool allocator
// (for example a Julia session whose CUDA.jl memory pool owns the device
// memory), or a solver loop with a fixed memory budget that must not grow
// or stall in cudaMalloc between steps.  For them this entry point assembles
// the CSR values of the stiffness into a device buffer they own, and stages
// the element matrices (the only scratch of the assembly) in a fixed,
// file-scope device array instead of a cudaMalloc'ed buffer.
//
// The array is FS_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads the
// library and stays there until the process exits.  Its device address is
// looked up once per device, on the first call made with that device
// current; make that first call before any stream capture.  Every call
// shares the one array and it keeps the contents of the last call: nothing
// in it has to start at zero (each call rewrites every element slot it later
// reads), but calls whose work overlaps on the GPU (two contexts or streams
// at once) race on it and must be serialised by the caller.
#include <mutex>

#include "fs_internal.cuh"

#define FS_NOALLOC_SCRATCH_BYTES (32u << 20)

namespace fs {

static __device__ __align__(256) unsigned char fs_noalloc_scratch[FS_NOALLOC_SCRATCH_BYTES];

// device address of the array, resolved once per device
static void *noalloc_scratch_ptr(fs_ctx *c, int *status)
{
    static std::mutex mu;
    static void *addr[64] = {nullptr};
    std::lock_guard<std::mutex> lock(mu);
    if (c->device < 0 || c->device >= 64) {
        *status = set_err(c, FS_ERR_UNSUPPORTED, "device index above 63");
        return nullptr;
    }
    if (!addr[c->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, fs_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            *status = set_err(c, FS_ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch array: ") +
                                                  cudaGetErrorString(e));
            return nullptr;
        }
        addr[c->device] = p;
    }
    *status = FS_OK;
    return addr[c->device];
}

}  // namespace fs

using namespace fs;

extern "C" int fs_stiffness_values_noalloc(fs_ctx *c, int precision, int64_t nrows, double *vals,
                                           int64_t vals_len)
{
    if (!c) return FS_ERR_BAD_INPUT;
    FS_CUDA(c, cudaSetDevice(c->device));
    if (precision != FS_FP64 && precision != FS_MIXED && precision != FS_MIXED_COMP)
        return set_err(c, FS_ERR_BAD_INPUT, "unknown precision");
    if (c->mesh.etype < 0 || !c->params_set || !c->dofs_ready)
        return set_err(c, FS_ERR_STATE, "mesh, parameters and dof numbering must be set first");
    if ((c->mesh.etype == FS_T3FFCOMP || c->mesh.etype == FS_Q4RSCOMP) && !c->mesh.groups)
        return set_err(c, FS_ERR_STATE, "layered FEMM without layups: call fs_layups_set first");
    if (!c->normals_ready)
        return set_err(c, FS_ERR_STATE, "associategeometry! has not been called (self._associatedgeometry == true)");
    if (c->pat.n != nrows || !c->pat.rowptr)
        return set_err(c, FS_ERR_STATE,
                       "no sparsity pattern for this matrix size: call fs_stiffness or fs_mass once at set-up");
    if (!vals) return set_err(c, FS_ERR_BAD_INPUT, "missing output buffer");
    if (vals_len < c->pat.nnz)
        return set_err(c, FS_ERR_BAD_INPUT, "output buffer shorter than the number of stored entries");
    const int nen = c->mesh.nen;
    const uint64_t per = (uint64_t)n_upper_blocks(nen) * 36 * entry_bytes(precision);
    const uint64_t need = per * (uint64_t)c->mesh.nelem;
    if (need > FS_NOALLOC_SCRATCH_BYTES) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "mesh too large for the allocation-free path: %lld elements need %llu bytes of element "
                 "matrices, the fixed scratch holds %u bytes (at most %llu elements)",
                 (long long)c->mesh.nelem, (unsigned long long)need, (unsigned)FS_NOALLOC_SCRATCH_BYTES,
                 (unsigned long long)(FS_NOALLOC_SCRATCH_BYTES / per));
        return set_err(c, FS_ERR_UNSUPPORTED, msg);
    }
    int st = FS_OK;
    void *scratch = noalloc_scratch_ptr(c, &st);
    if (!scratch) return st;
    FS_TRY(launch_elements_to(c, precision, scratch));
    FS_TRY(launch_gather_from(c, precision, scratch, vals));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    if (bits & DEV_SINGULAR) return set_err(c, FS_ERR_SINGULAR_METRIC, "Singular metric matrix in _gradN_e!");
    if (bits) return set_err(c, FS_ERR_BAD_INPUT, "invalid input detected on the device");
    return FS_OK;
}

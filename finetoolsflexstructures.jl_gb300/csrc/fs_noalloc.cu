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
// looked up when a context is created (fs_ctx_create, with the context's
// device current), so the library's device code and the array are loaded
// then, not on the first allocation-free call; that call and every later one
// only use the stored address.  Every call shares the one array and it keeps
// the contents of the last call: nothing in it has to start at zero (each
// call rewrites every element slot it later reads), but calls whose work
// overlaps on the GPU (two contexts or streams at once) race on it and must
// be serialised by the caller.
#include "fs_internal.cuh"

#define FS_NOALLOC_SCRATCH_BYTES (32u << 20)

namespace fs {

static __device__ __align__(256) unsigned char fs_noalloc_scratch[FS_NOALLOC_SCRATCH_BYTES];

// The array's address in the CUDA context current at context creation (the
// context every buffer of `c` lives in).  A failed lookup is recorded, not
// fatal: only the allocation-free entry point needs the address.
void noalloc_setup(fs_ctx *c)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, fs_noalloc_scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c->noalloc_scratch = nullptr;
        c->noalloc_err = std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e);
        return;
    }
    c->noalloc_scratch = p;
    c->noalloc_err.clear();
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
    // shell mesh (beams are rejected), parameters, dofs and layups
    FS_TRY(check_ready(c));
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
    if (!c->noalloc_scratch) return set_err(c, FS_ERR_CUDA, c->noalloc_err);
    FS_TRY(launch_elements_to(c, precision, c->noalloc_scratch));
    FS_TRY(launch_gather_from(c, precision, c->noalloc_scratch, vals));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    return status_to_code(c, bits);
}

// Symbolic phase: mesh preparation, node-to-element adjacency and the CSR
// sparsity pattern of the assembled matrix.
//
// The pattern depends only on the connectivity, the dof numbering and the
// matrix size, so it is built once per mesh and reused by every numeric
// assembly.  Its semantics are those of Julia's sparse(I, J, V) over the
// element dof pairs (FinEtools SysmatAssemblerSparse, src/AssemblyModule.jl):
// row d holds every column that shares an element with it, sorted.  Rows are
// produced per node: all six dofs of a node share one sorted column list.
#include <algorithm>
#include <vector>

#include "fs_internal.cuh"

namespace fs {

static const int SCAN_TPB = 256;
static const int SCAN_ITEMS = 4;
static const int SCAN_CHUNK = SCAN_TPB * SCAN_ITEMS;

// ---------------------------------------------------------------------------
// exclusive scan of int64 (out has n + 1 entries, out[n] = total)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t warp_incl_scan(int64_t v)
{
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += u;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total
__device__ int64_t block_excl_scan(int64_t v, int64_t &excl)
{
    __shared__ int64_t wsum[SCAN_TPB / 32];
    int64_t inc = warp_incl_scan(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < SCAN_TPB / 32 ? wsum[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < SCAN_TPB / 32) wsum[lane] = s;
    }
    __syncthreads();
    int64_t before = w ? wsum[w - 1] : 0;
    int64_t total = wsum[SCAN_TPB / 32 - 1];
    excl = before + inc - v;
    __syncthreads();
    return total;
}

__global__ void k_chunk_sums(const int64_t *in, int64_t n, int64_t *sums)
{
    int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
    int64_t s = 0;
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t k = base + (int64_t)i * SCAN_TPB + threadIdx.x;
        if (k < n) s += in[k];
    }
    int64_t ex;
    int64_t tot = block_excl_scan(s, ex);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block: exclusive scan of the chunk sums in place, total at [nchunks]
__global__ void k_scan_sums(int64_t *sums, int64_t nchunks)
{
    int64_t carry = 0;
    for (int64_t base = 0; base < nchunks; base += SCAN_TPB) {
        int64_t k = base + threadIdx.x;
        int64_t v = k < nchunks ? sums[k] : 0;
        int64_t ex;
        int64_t tot = block_excl_scan(v, ex);
        if (k < nchunks) sums[k] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nchunks] = carry;
}

__global__ void k_chunk_scan(const int64_t *in, int64_t n, const int64_t *sums, int64_t *out)
{
    int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t k = base + i;
        v[i] = k < n ? in[k] : 0;
        s += v[i];
    }
    int64_t ex;
    block_excl_scan(s, ex);
    int64_t run = sums[blockIdx.x] + ex;
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t k = base + i;
        if (k < n) out[k] = run;
        run += v[i];
    }
}

__global__ void k_set_total(int64_t *out, int64_t n, const int64_t *sums, int64_t nchunks)
{
    out[n] = sums[nchunks];
}

int exclusive_scan_i64(fs_ctx *c, const int64_t *in, int64_t *out, int64_t n, int64_t *total)
{
    int64_t nchunks = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (nchunks == 0) nchunks = 1;
    FS_TRY(ensure_scratch(c, sizeof(int64_t) * (nchunks + 1)));
    int64_t *sums = (int64_t *)c->scratch;
    k_chunk_sums<<<(unsigned)nchunks, SCAN_TPB, 0, c->stream>>>(in, n, sums);
    k_scan_sums<<<1, SCAN_TPB, 0, c->stream>>>(sums, nchunks);
    k_chunk_scan<<<(unsigned)nchunks, SCAN_TPB, 0, c->stream>>>(in, n, sums, out);
    k_set_total<<<1, 1, 0, c->stream>>>(out, n, sums, nchunks);
    FS_CUDA(c, cudaGetLastError());
    if (total) {
        FS_CUDA(c, cudaMemcpyAsync(total, out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        FS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return FS_OK;
}

// ---------------------------------------------------------------------------
// mesh preparation
// ---------------------------------------------------------------------------
__global__ void k_prepare_conn(int64_t nelem, int nen, int64_t nnodes, const int64_t *conn_raw,
                               const int64_t *order, int32_t *conn, int32_t *elem_of_rank,
                               int32_t *seen, int *status)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nelem) return;
    int64_t e = order ? order[r] - 1 : r;
    if (e < 0 || e >= nelem) {
        atomicOr(status, DEV_BAD_ORDER);
        e = 0;
    } else if (order && atomicAdd(&seen[e], 1) != 0) {
        atomicOr(status, DEV_BAD_ORDER);
    }
    elem_of_rank[r] = (int32_t)e;
    for (int a = 0; a < nen; a++) {
        int64_t node = conn_raw[e * nen + a] - 1;
        if (node < 0 || node >= nnodes) {
            atomicOr(status, DEV_BAD_CONN);
            node = 0;
        }
        conn[r * nen + a] = (int32_t)node;
    }
}

__global__ void k_prepare_dof(int64_t m, const int64_t *dof_raw, int32_t *dof, int *status)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int64_t v = dof_raw[i];
    if (v < 1 || v > 0x7fffffffLL) {
        atomicOr(status, DEV_BAD_DOF);
        v = 0x7fffffff;
    }
    dof[i] = (int32_t)v;
}

static unsigned nblk(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

int launch_prepare_mesh(fs_ctx *c, const int64_t *d_conn_raw, const int64_t *d_order_raw,
                        const int64_t *d_dof_raw)
{
    MeshDev &m = c->mesh;
    int32_t *seen = nullptr;
    if (d_order_raw) {
        FS_TRY(dalloc(c, &seen, (size_t)m.nelem));
        FS_CUDA(c, cudaMemsetAsync(seen, 0, sizeof(int32_t) * m.nelem, c->stream));
    }
    if (m.nelem > 0)
        k_prepare_conn<<<nblk(m.nelem, 256), 256, 0, c->stream>>>(m.nelem, m.nen, m.nnodes, d_conn_raw,
                                                                  d_order_raw, m.conn, m.elem_of_rank, seen,
                                                                  c->d_status);
    if (d_dof_raw && m.nnodes)
        k_prepare_dof<<<nblk(6 * m.nnodes, 256), 256, 0, c->stream>>>(6 * m.nnodes, d_dof_raw, m.dof,
                                                                      c->d_status);
    FS_CUDA(c, cudaGetLastError());
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    if (seen) cudaFree(seen);
    if (bits & DEV_BAD_CONN) return set_err(c, FS_ERR_BAD_INPUT, "connectivity refers to a node outside 1..nnodes");
    if (bits & DEV_BAD_ORDER) return set_err(c, FS_ERR_BAD_INPUT, "assembly order is not a permutation of 1..nelem");
    if (bits & DEV_BAD_DOF) return set_err(c, FS_ERR_BAD_INPUT, "dof numbers must be in 1..2^31-1");
    return FS_OK;
}

int launch_prepare_dofs(fs_ctx *c, const int64_t *d_dof_raw)
{
    MeshDev &m = c->mesh;
    if (m.nnodes)
        k_prepare_dof<<<nblk(6 * m.nnodes, 256), 256, 0, c->stream>>>(6 * m.nnodes, d_dof_raw, m.dof, c->d_status);
    FS_CUDA(c, cudaGetLastError());
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    if (bits & DEV_BAD_DOF) return set_err(c, FS_ERR_BAD_INPUT, "dof numbers must be in 1..2^31-1");
    return FS_OK;
}

// ---------------------------------------------------------------------------
// node -> element adjacency (ascending assembly rank)
// ---------------------------------------------------------------------------
__global__ void k_count_pairs(int64_t nelem, int nen, const int32_t *conn, int64_t *cnt)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nelem * nen) return;
    atomicAdd((unsigned long long *)&cnt[conn[i]], 1ull);
}

__global__ void k_fill_pairs(int64_t nelem, int nen, const int32_t *conn, const int64_t *pp,
                             int64_t *fill, int32_t *pair_e)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nelem * nen) return;
    int node = conn[i];
    int64_t r = i / nen;
    int a = (int)(i - r * nen);
    int64_t s = (int64_t)atomicAdd((unsigned long long *)&fill[node], 1ull);
    pair_e[pp[node] + s] = (int32_t)((r << 2) | a);
}

__global__ void k_sort_pairs(int64_t nnodes, const int64_t *pp, int32_t *pair_e, int *status)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nnodes) return;
    int64_t b = pp[r], e = pp[r + 1];
    if (e - b > MAX_PAIRS_PER_NODE) atomicOr(status, DEV_VALENCE);
    for (int64_t i = b + 1; i < e; i++) {
        int32_t v = pair_e[i];
        int64_t j = i - 1;
        while (j >= b && pair_e[j] > v) {
            pair_e[j + 1] = pair_e[j];
            j--;
        }
        pair_e[j + 1] = v;
    }
}

__global__ void k_elem_pair(int64_t npairs, int nen, const int32_t *pair_e, int32_t *elem_pair)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int32_t v = pair_e[p];
    elem_pair[(int64_t)(v >> 2) * nen + (v & 3)] = (int32_t)p;
}

int build_adjacency(fs_ctx *c)
{
    MeshDev &m = c->mesh;
    int64_t nn = m.nnodes, ne = m.nelem;
    m.npairs = ne * m.nen;
    FS_TRY(dalloc(c, &m.pp, (size_t)nn + 1));
    FS_TRY(dalloc(c, &m.pair_e, (size_t)m.npairs));
    FS_TRY(dalloc(c, &m.elem_pair, (size_t)m.npairs));
    int64_t *cnt = nullptr;
    FS_TRY(dalloc(c, &cnt, (size_t)nn));
    FS_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * nn, c->stream));
    if (m.npairs) k_count_pairs<<<nblk(m.npairs, 256), 256, 0, c->stream>>>(ne, m.nen, m.conn, cnt);
    FS_TRY(exclusive_scan_i64(c, cnt, m.pp, nn, nullptr));
    FS_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * nn, c->stream));
    if (m.npairs) k_fill_pairs<<<nblk(m.npairs, 256), 256, 0, c->stream>>>(ne, m.nen, m.conn, m.pp, cnt, m.pair_e);
    if (nn) k_sort_pairs<<<nblk(nn, 128), 128, 0, c->stream>>>(nn, m.pp, m.pair_e, c->d_status);
    if (m.npairs) k_elem_pair<<<nblk(m.npairs, 256), 256, 0, c->stream>>>(m.npairs, m.nen, m.pair_e, m.elem_pair);
    FS_CUDA(c, cudaGetLastError());
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    cudaFree(cnt);
    if (bits & DEV_VALENCE)
        return set_err(c, FS_ERR_UNSUPPORTED, "more than 64 elements meet at one node");
    return FS_OK;
}

// ---------------------------------------------------------------------------
// neighbour lists and per-node column layout
// ---------------------------------------------------------------------------
// Sorted unique neighbour nodes of node r, in a thread-local buffer.
__device__ int node_neighbors(int64_t r, int nen, const int64_t *pp, const int32_t *pair_e,
                              const int32_t *conn, int32_t *buf)
{
    int64_t b = pp[r], e = pp[r + 1];
    if (e - b > MAX_PAIRS_PER_NODE) e = b + MAX_PAIRS_PER_NODE;
    int n = 0;
    for (int64_t p = b; p < e; p++) {
        int64_t rank = pair_e[p] >> 2;
        for (int k = 0; k < nen; k++) {
            int32_t v = conn[rank * nen + k];
            // insertion into sorted unique buffer
            int j = n - 1;
            bool dup = false;
            while (j >= 0 && buf[j] >= v) {
                if (buf[j] == v) { dup = true; break; }
                j--;
            }
            if (dup) continue;
            for (int q = n; q > j + 1; q--) buf[q] = buf[q - 1];
            buf[j + 1] = v;
            n++;
        }
    }
    return n;
}

__global__ void k_count_nbrs(int64_t nnodes, int nen, const int64_t *pp, const int32_t *pair_e,
                             const int32_t *conn, int64_t *cnt, int *status)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nnodes) return;
    int32_t buf[MAX_PAIRS_PER_NODE * 4];
    int n = node_neighbors(r, nen, pp, pair_e, conn, buf);
    if (n > MAX_NBRS) atomicOr(status, DEV_NEIGHBORS);
    cnt[r] = n;
}

__global__ void k_fill_nbrs(int64_t nnodes, int nen, int64_t n_mat, const int64_t *pp,
                            const int32_t *pair_e, const int32_t *conn, const int32_t *dof,
                            const int64_t *nbr_off, int32_t *nbr, uint32_t *pair_slots,
                            int16_t *colpos, uint16_t *colsrc, int32_t *rowlen, uint16_t *sl_off,
                            uint16_t *sl_ent)
{
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nnodes) return;
    int32_t buf[MAX_PAIRS_PER_NODE * 4];
    int n = node_neighbors(r, nen, pp, pair_e, conn, buf);
    if (n > MAX_NBRS) n = MAX_NBRS;
    int64_t off = nbr_off[r];
    for (int s = 0; s < n; s++) nbr[off + s] = buf[s];
    // slots of each element node in this node's neighbour list
    for (int64_t p = pp[r]; p < pp[r + 1]; p++) {
        int64_t rank = pair_e[p] >> 2;
        uint32_t packed = 0;
        for (int k = 0; k < nen; k++) {
            int32_t v = conn[rank * nen + k];
            int lo = 0, hi = n - 1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (buf[mid] < v) lo = mid + 1; else hi = mid;
            }
            packed |= (uint32_t)(lo & 0xff) << (8 * k);
        }
        pair_slots[p] = packed;
    }
    // contribution lists per neighbour slot (ascending pair order)
    {
        const int64_t p0 = pp[r];
        const int np = (int)min((int64_t)MAX_PAIRS_PER_NODE, pp[r + 1] - p0);
        uint16_t *ent = sl_ent + p0 * nen;
        int w = 0;
        for (int s = 0; s < n; s++) {
            sl_off[off + s] = (uint16_t)w;
            for (int q = 0; q < np; q++) {
                const uint32_t packed = pair_slots[p0 + q];
                const int aq = pair_e[p0 + q] & 3;
                for (int b = 0; b < nen; b++)
                    if ((int)((packed >> (8 * b)) & 0xffu) == s)
                        ent[w++] = (uint16_t)(q | (b << 6) | ((b < aq ? 1 : 0) << 8));
            }
        }
    }
    // column positions: rank of each valid column dof among the node's columns
    int L = 0;
    if (6 * n <= MAX_PAIRS_PER_NODE * 4) {
        // the neighbours' dofs read once into a local list (it overwrites the
        // neighbour list, already stored: going backwards, buf[s] is read
        // before cd[6 s ..] is written), excluded dofs marked 0, then ranked
        int32_t *cd = buf;
        for (int s = n - 1; s >= 0; s--) {
            const int32_t node = buf[s];
            for (int k = 5; k >= 0; k--) {
                const int32_t v = dof[(int64_t)k * nnodes + node];
                cd[6 * s + k] = v <= n_mat ? v : 0;
            }
        }
        // the usual numbering (node-major, the neighbours sorted) lists the
        // kept dofs in increasing order: their rank is their running count;
        // any other numbering is ranked by counting
        bool sorted = true;
        int32_t prev = 0;
        for (int q = 0; q < 6 * n; q++) {
            const int32_t v = cd[q];
            if (v != 0) {
                sorted &= v > prev;
                prev = v;
                L++;
            }
        }
        int run = 0;
        for (int q = 0; q < 6 * n; q++) {
            const int32_t v = cd[q];
            int16_t pos = -1;
            if (v != 0) {
                if (sorted) {
                    pos = (int16_t)run++;
                } else {
                    int cntless = 0;
                    for (int q2 = 0; q2 < 6 * n; q2++) cntless += (cd[q2] != 0) & (cd[q2] < v);
                    pos = (int16_t)cntless;
                }
            }
            colpos[off * 6 + q] = pos;
            if (pos >= 0) colsrc[off * 6 + pos] = (uint16_t)q;
        }
    } else {
        for (int s = 0; s < n; s++)
            for (int k = 0; k < 6; k++) L += (dof[(int64_t)k * nnodes + buf[s]] <= n_mat);
        for (int s = 0; s < n; s++)
            for (int k = 0; k < 6; k++) {
                int32_t v = dof[(int64_t)k * nnodes + buf[s]];
                int16_t pos = -1;
                if (v <= n_mat) {
                    int cntless = 0;
                    for (int s2 = 0; s2 < n; s2++)
                        for (int k2 = 0; k2 < 6; k2++) {
                            int32_t w = dof[(int64_t)k2 * nnodes + buf[s2]];
                            cntless += (w <= n_mat) & (w < v);
                        }
                    pos = (int16_t)cntless;
                }
                colpos[off * 6 + s * 6 + k] = pos;
                if (pos >= 0) colsrc[off * 6 + pos] = (uint16_t)(s * 6 + k);
            }
    }
    rowlen[r] = L;
}

// Per (node r, neighbour slot) the data the gather needs to compute each
// node-block pair once: a block (r, s) with r < s is summed by r's warp,
// which also writes it transposed into s's rows, when both nodes take the
// gather's register path (a row of at most 64 or 128 positions, fewer than 32
// neighbour slots, some row in the matrix); s's warp then skips it.  Per slot
// one word: m << 4 | flags, flags bit 0 s < r, bit 1 s > r, bit 2 s qualifies
// at 64 positions, bit 3 at 128; m, for s > r, the slot of r in s's list as an
// index into the neighbour entries (6 m indexes colpos: the column positions
// of r's dofs in s's rows).  lc: the row positions r's warp sums in the
// register path of rows up to 64 positions (its row length less the columns
// of lower neighbours that qualify there; 0 without rows).
__global__ void k_slot_mirror(int64_t nnodes, int64_t n_mat, const int32_t *dof, const int64_t *nbr_off,
                              const int32_t *nbr, const int32_t *rowlen, uint32_t *mir, int32_t *lc)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nnodes) return;
    const int64_t off = nbr_off[r], n = nbr_off[r + 1] - off;
    bool rrow = false;
    for (int k = 0; k < 6; k++) rrow |= dof[(int64_t)k * nnodes + r] <= n_mat;
    const bool rq = rrow && n < 32 && rowlen[r] <= 64;
    int cnt = rrow ? rowlen[r] : 0;
    for (int64_t sl = 0; sl < n; sl++) {
        const int32_t s = nbr[off + sl];
        const int64_t so = nbr_off[s], sn = nbr_off[s + 1] - so;
        int nfree = 0;
        for (int k = 0; k < 6; k++) nfree += dof[(int64_t)k * nnodes + s] <= n_mat;
        const bool anyrow = nfree > 0;
        const int L = rowlen[s];
        const bool q = anyrow && sn < 32;
        if (rq && s < r && q && L <= 64) cnt -= nfree;
        const uint32_t f = (s < r ? 1u : 0u) | (s > r ? 2u : 0u) | (q && L <= 64 ? 4u : 0u) | (q && L <= 128 ? 8u : 0u);
        uint32_t mv = 0;
        if (s > r) {
            int64_t lo = 0, hi = sn - 1;  // r in s's sorted list
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (nbr[so + mid] < r) lo = mid + 1; else hi = mid;
            }
            mv = (uint32_t)(so + lo);
        }
        mir[off + sl] = mv << 4 | f;
    }
    lc[r] = cnt;
}

// *out = max(v[0..n)) (out zeroed before; values are non-negative)
__global__ void k_max_i32(int64_t n, const int32_t *v, int32_t *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t x = i < n ? v[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
    if ((threadIdx.x & 31) == 0 && x > 0) atomicMax(out, x);
}

__global__ void k_row_lengths(int64_t nnodes, int64_t n_mat, const int32_t *dof, const int32_t *rowlen,
                              int64_t *rl, int32_t *owner_cnt, int *status)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nnodes) return;
    int64_t r = i % nnodes;
    int32_t d = dof[i];
    if (d <= n_mat) {
        if (atomicAdd(&owner_cnt[d - 1], 1) != 0) atomicOr(status, DEV_BAD_DOF);
        rl[d - 1] = rowlen[r];
    }
}

// One warp per node: position j of the node's rows holds the column of
// (neighbour slot, component) colsrc[j]; the six rows share it, so each row
// is written as one contiguous run.
__global__ void k_fill_colidx(int64_t nnodes, int64_t n_mat, const int32_t *dof, const int64_t *nbr_off,
                              const int32_t *nbr, const uint16_t *colsrc, const int32_t *rowlen,
                              const int64_t *rowptr, int32_t *colidx)
{
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= nnodes) return;
    const int64_t off = nbr_off[r];
    const int L = rowlen[r];
    int64_t base[6];
#pragma unroll
    for (int kr = 0; kr < 6; kr++) {
        const int32_t d = dof[(int64_t)kr * nnodes + r];
        base[kr] = d <= n_mat ? rowptr[d - 1] : -1;
    }
    for (int j = lane; j < L; j += 32) {
        const int cs = colsrc[off * 6 + j];
        const int s = cs / 6, k = cs - 6 * s;
        const int32_t col = dof[(int64_t)k * nnodes + nbr[off + s]] - 1;
#pragma unroll
        for (int kr = 0; kr < 6; kr++)
            if (base[kr] >= 0) colidx[base[kr] + j] = col;
    }
}

__global__ void k_diag_pattern(int64_t n, int64_t *rowptr, int32_t *colidx)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) rowptr[i] = i;
    if (i < n) colidx[i] = (int32_t)i;
}

int build_pattern(fs_ctx *c, int64_t n)
{
    MeshDev &m = c->mesh;
    PatternDev &P = c->pat;
    if (P.n == n && P.rowptr) return FS_OK;
    int64_t nn = m.nnodes;
    if (n > 0x7fffffffLL) return set_err(c, FS_ERR_UNSUPPORTED, "matrix size above 2^31-1");
    int64_t *cnt = nullptr;
    FS_TRY(grow(c, &P.tmp_cnt, &P.cap_tmp_cnt, (size_t)std::max<int64_t>(nn, n)));
    cnt = P.tmp_cnt;
    if (nn) k_count_nbrs<<<nblk(nn, 128), 128, 0, c->stream>>>(nn, m.nen, m.pp, m.pair_e, m.conn, cnt, c->d_status);
    FS_TRY(grow(c, &P.nbr_off, &P.cap_nbr_off, (size_t)nn + 1));
    int64_t nbr_total = 0;
    FS_TRY(exclusive_scan_i64(c, cnt, P.nbr_off, nn, &nbr_total));
    int bits = 0;
    FS_TRY(read_status(c, &bits));
    if (bits & DEV_NEIGHBORS) {
        return set_err(c, FS_ERR_UNSUPPORTED, "more than 255 neighbour nodes at one node");
    }
    FS_TRY(grow(c, &P.nbr, &P.cap_nbr, (size_t)nbr_total));
    FS_TRY(grow(c, &P.pair_slots, &P.cap_pair_slots, (size_t)m.npairs));
    FS_TRY(grow(c, &P.colpos, &P.cap_colpos, (size_t)nbr_total * 6));
    FS_TRY(grow(c, &P.colsrc, &P.cap_colsrc, (size_t)nbr_total * 6));
    FS_TRY(grow(c, &P.rowlen, &P.cap_rowlen, (size_t)nn));
    FS_TRY(grow(c, &P.sl_off, &P.cap_sl_off, (size_t)nbr_total));
    FS_TRY(grow(c, &P.sl_ent, &P.cap_sl_ent, (size_t)(m.npairs * m.nen)));
    if (nn)
        k_fill_nbrs<<<nblk(nn, 128), 128, 0, c->stream>>>(nn, m.nen, n, m.pp, m.pair_e, m.conn, m.dof, P.nbr_off,
                                                         P.nbr, P.pair_slots, P.colpos, P.colsrc, P.rowlen,
                                                         P.sl_off, P.sl_ent);
    // row lengths by dof
    int32_t *owner = nullptr;
    FS_TRY(grow(c, &P.tmp_owner, &P.cap_tmp_owner, (size_t)n));
    owner = P.tmp_owner;
    FS_CUDA(c, cudaMemsetAsync(owner, 0, sizeof(int32_t) * std::max<int64_t>(n, 1), c->stream));
    FS_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * std::max<int64_t>(n, 1), c->stream));
    if (nn) k_row_lengths<<<nblk(6 * nn, 256), 256, 0, c->stream>>>(nn, n, m.dof, P.rowlen, cnt, owner, c->d_status);
    // longest row (selects the gather variant): reduced on the device, read
    // back with the scan total
    int32_t *d_max = reinterpret_cast<int32_t *>(owner);  // owner counts are consumed by k_row_lengths
    FS_CUDA(c, cudaMemsetAsync(d_max, 0, sizeof(int32_t), c->stream));
    if (nn) k_max_i32<<<nblk(nn, 256), 256, 0, c->stream>>>(nn, P.rowlen, d_max);
    int32_t mx = 0;
    FS_CUDA(c, cudaMemcpyAsync(&mx, d_max, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    FS_TRY(grow(c, &P.rowptr, &P.cap_rowptr, (size_t)n + 1));
    int64_t nnz = 0;
    FS_TRY(exclusive_scan_i64(c, cnt, P.rowptr, n, &nnz));
    P.maxlen = mx;  // the scan's read-back synchronised the stream
    FS_TRY(read_status(c, &bits));
    if (bits & DEV_BAD_DOF) return set_err(c, FS_ERR_BAD_INPUT, "two dofs share one dof number");
    FS_TRY(grow(c, &P.colidx, &P.cap_colidx, (size_t)nnz));
    if (nn)
        k_fill_colidx<<<nblk(nn * 32, 256), 256, 0, c->stream>>>(nn, n, m.dof, P.nbr_off, P.nbr, P.colsrc,
                                                                  P.rowlen, P.rowptr, P.colidx);
    // node-block pairs summed once (neighbour entry indices fit 28 bits)
    P.maxlc = mx;
    if (nbr_total < (1LL << 28)) {
        FS_TRY(grow(c, &P.sl_mir, &P.cap_sl_mir, (size_t)nbr_total));
        FS_TRY(grow(c, &P.lc, &P.cap_lc, (size_t)nn));
        if (nn) {
            k_slot_mirror<<<nblk(nn, 128), 128, 0, c->stream>>>(nn, n, m.dof, P.nbr_off, P.nbr, P.rowlen, P.sl_mir,
                                                               P.lc);
            // the longest summed row (selects the one-column variant of the gather)
            FS_CUDA(c, cudaMemsetAsync(d_max, 0, sizeof(int32_t), c->stream));
            k_max_i32<<<nblk(nn, 256), 256, 0, c->stream>>>(nn, P.lc, d_max);
            FS_CUDA(c, cudaMemcpyAsync(&mx, d_max, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
        }
        P.sym = true;
    } else {
        P.sym = false;
    }
    FS_TRY(grow(c, &P.diag_rowptr, &P.cap_diag_rowptr, (size_t)n + 1));
    FS_TRY(grow(c, &P.diag_colidx, &P.cap_diag_colidx, (size_t)n));
    k_diag_pattern<<<nblk(n + 1, 256), 256, 0, c->stream>>>(n, P.diag_rowptr, P.diag_colidx);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (P.sym && nn) P.maxlc = mx;
    P.n = n;
    P.nnz = nnz;
    return FS_OK;
}

// ---------------------------------------------------------------------------
// dropping exact zeros (FinEtools SysmatAssemblerSparseSymm: S + S^T keeps
// only nonzero results)
// ---------------------------------------------------------------------------
__global__ void k_count_nonzero(int64_t n, const int64_t *rowptr, const double *vals, int64_t *cnt)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t s = 0;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) s += (vals[k] != 0.0);
    cnt[i] = s;
}

__global__ void k_compact(int64_t n, const int64_t *rowptr, const int32_t *colidx, const double *vals,
                          const int64_t *nrowptr, int32_t *ncol, double *nval)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t w = nrowptr[i];
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (vals[k] != 0.0) {
            ncol[w] = colidx[k];
            nval[w] = vals[k];
            w++;
        }
}

int compact_zeros(fs_ctx *c, int64_t n, const int64_t *rowptr, const int32_t *colidx, const double *vals,
                  int64_t nnz)
{
    int64_t *cnt = nullptr;
    FS_TRY(dalloc(c, &cnt, (size_t)n));
    if (n) k_count_nonzero<<<nblk(n, 256), 256, 0, c->stream>>>(n, rowptr, vals, cnt);
    FS_TRY(dalloc(c, &c->cmp_rowptr, (size_t)n + 1));
    int64_t nnz2 = 0;
    FS_TRY(exclusive_scan_i64(c, cnt, c->cmp_rowptr, n, &nnz2));
    cudaFree(cnt);
    if (nnz2 == nnz) {
        // nothing to drop: keep the arrays as they are
        c->mat_rowptr = rowptr;
        c->mat_colidx = colidx;
        c->mat_nnz = nnz;
        return FS_OK;
    }
    if ((size_t)nnz2 > c->cmp_cap || !c->cmp_colidx) {
        FS_TRY(dalloc(c, &c->cmp_colidx, (size_t)nnz2));
        FS_TRY(dalloc(c, &c->cmp_vals, (size_t)nnz2));
        c->cmp_cap = (size_t)nnz2;
    }
    if (n) k_compact<<<nblk(n, 256), 256, 0, c->stream>>>(n, rowptr, colidx, vals, c->cmp_rowptr, c->cmp_colidx, c->cmp_vals);
    FS_CUDA(c, cudaGetLastError());
    FS_CUDA(c, cudaMemcpyAsync(c->vals, c->cmp_vals, sizeof(double) * nnz2, cudaMemcpyDeviceToDevice, c->stream));
    FS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->mat_rowptr = c->cmp_rowptr;
    c->mat_colidx = c->cmp_colidx;
    c->mat_nnz = nnz2;
    return FS_OK;
}

}  // namespace fs

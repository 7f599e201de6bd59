"""Matrix comparisons shared by the GPU parity tests."""
import numpy as np


def relmax(A, B):
    """max |A - B| / max |B|; sparse operands stay sparse."""
    import scipy.sparse as sp
    if sp.issparse(A) or sp.issparse(B):
        A = sp.csr_matrix(A)
        B = sp.csr_matrix(B)
        D = A - B
        num = np.abs(D.data).max() if D.nnz else 0.0
        return num / np.abs(B.data).max()
    A = np.asarray(A)
    B = np.asarray(B)
    return np.abs(A - B).max() / np.abs(B).max()


def same_pattern(A, B):
    A = A.tocsc()
    B = B.tocsc()
    A.has_sorted_indices and B.has_sorted_indices
    return (A.shape == B.shape and np.array_equal(A.indptr, B.indptr)
            and np.array_equal(A.indices, B.indices))


def same_pattern_modulo_cancellation(A, B, rel=1e-14):
    """Patterns of two zero-dropping (SysmatAssemblerSparseSymm) results: an
    entry may be stored in only one of them when its exact value is zero and
    one operation order cancels it exactly while the other leaves round-off;
    such entries must be below `rel` times the largest entry in both."""
    A = A.tocsc()
    B = B.tocsc()
    if A.shape != B.shape:
        return False
    PA = (A != 0).astype(np.int8)
    PB_ = (B != 0).astype(np.int8)
    D = (PA - PB_).tocoo()
    scale = max(abs(A).max(), abs(B).max())
    for r, c in zip(D.row[D.data != 0], D.col[D.data != 0]):
        if abs(A[r, c]) > rel * scale or abs(B[r, c]) > rel * scale:
            return False
    return True


def entrywise_errors(A, B, floor=1e-12):
    """Entrywise comparisons of A against the reference B on B's pattern:
    relmax = max |A - B| / max |B|; scaled = max |A_ij - B_ij| / sqrt(|B_ii B_jj|)
    (the natural scale of an entry of a positive semi-definite matrix, which
    bounds it); entrywise = max |A_ij - B_ij| / |B_ij| over the entries with
    |B_ij| > floor max |B| (entries that are small only through cancellation
    carry the rounding of the large terms they are summed from)."""
    import scipy.sparse as sp
    A = sp.csr_matrix(A)
    B = sp.csr_matrix(B)
    A.sort_indices()
    B.sort_indices()
    Bc = B.tocoo()
    if (A.shape == B.shape and np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)):
        dv = A.data - B.data
    else:
        dv = np.asarray((A - B)[Bc.row, Bc.col]).ravel()
    mx = np.abs(B.data).max()
    d = np.abs(B.diagonal())
    den = np.sqrt(d[Bc.row] * d[Bc.col])
    ok = den > 0
    big = np.abs(Bc.data) > floor * mx
    return {"relmax": float(np.abs(dv).max() / mx),
            "scaled": float((np.abs(dv[ok]) / den[ok]).max()) if ok.any() else 0.0,
            "entrywise": float((np.abs(dv[big]) / np.abs(Bc.data[big])).max()) if big.any() else 0.0}

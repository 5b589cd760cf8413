"""numpy restatement of plantFEM's LOBPCG_CRS (TEST INFRASTRUCTURE ONLY).

Follows ``src/SparseClass/SparseClass.f90:2008-2239`` step by step, with
``GramSchmidt`` (``:2243-2275``) restated literally and LAPACK ``DSPGVD``
(ITYPE=1, JOBZ='V', UPLO='U'; ``:2279-2351``) replaced by
``scipy.linalg.eigh(a, b, type=1)``, which solves the same generalized
symmetric-definite problem (ascending eigenvalues, B-normalised vectors).
DSPGVD is an un-vendored LAPACK dependency (linked as ``-llapack`` in the
reference's Makefile:8, no pinned version); scipy's bundled LAPACK stands in.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def gram_schmidt(V: np.ndarray) -> np.ndarray:
    """GramSchmidt (SparseClass.f90:2243-2275): column-sequential modified GS,
    zero columns skipped, each column normalised after projection.  Runs the
    compiled restatement (``orc_gram_schmidt``, OpenMP) when the oracle
    library is built, else :func:`gram_schmidt_numpy`."""
    try:
        from . import lib
        L = lib()
    except Exception:  # library not built: the numpy loop
        return gram_schmidt_numpy(V)
    if np.asarray(V).flags.f_contiguous and not np.asarray(V).flags.c_contiguous:
        out = np.array(V, dtype=np.float64, order="F", copy=True)
        L.orc_gram_schmidt(out.shape[0], out.shape[1], out.ctypes.data)
    else:  # row-major: transposed inside the library (a numpy transpose copy is slow)
        out = np.array(V, dtype=np.float64, order="C", copy=True)
        L.orc_gram_schmidt_rm(out.shape[0], out.shape[1], out.ctypes.data, None)
    return out


def _gram_schmidt_inplace(V: np.ndarray, scratch: np.ndarray) -> None:
    """gram_schmidt on a C-contiguous V in place (compiled, with a reused scratch)."""
    from . import lib
    lib().orc_gram_schmidt_rm(V.shape[0], V.shape[1], V.ctypes.data, scratch.ctypes.data)


def _mm_into(A, X, out):
    if hasattr(A, "matmul_into"):
        A.matmul_into(X, out)
    else:
        out[...] = A @ X


def gram_schmidt_numpy(V: np.ndarray) -> np.ndarray:
    """The same in numpy, one column operation at a time."""
    out = np.asfortranarray(V, dtype=np.float64).copy(order="F")  # contiguous columns
    m = out.shape[1]
    for i in range(m):
        viold = out[:, i].copy()
        if np.dot(viold, viold) == 0.0:
            continue
        for j in range(i):
            nai = np.dot(out[:, j], viold)
            viold = viold - nai * out[:, j]
        out[:, i] = viold / np.sqrt(np.dot(viold, viold))
    return out


def lapack_eig(A, B):
    """LAPACK_EIG_DENSE via DSPGVD (ascending eigenvalues, B-orthonormal vectors)."""
    w, Z = sla.eigh(0.5 * (A + A.T), 0.5 * (B + B.T), type=1)
    return Z, w


def lobpcg_crs(A, B, m: int, max_itr: int = 100000, tol: float = 1e-6, X_init=None, seed: int = 0,
               return_iters: bool = False, progress=None):
    """LOBPCG_CRS(A, B, lambda, X, m, MAX_ITR, TOL, X_init) with A, B scipy sparse.

    Convergence test as the reference: max|R| / max|R at iteration 1| < TOL
    (SparseClass.f90:2218-2234).  ``progress(it, ratio, lam, R, BX)``, if
    given, is called after every iteration (R and BX: the block's residuals and
    B X); a true return ends the iteration there (a caller that needs only some
    of the m pairs converged).  The random start (``random%randn`` is
    uniform, RandomClass.f90:265-283) uses a seeded numpy generator here.
    """
    n = A.shape[0]
    rng = np.random.default_rng(seed)
    X = rng.random((n, m)) if X_init is None else np.array(X_init, dtype=np.float64)
    X = X / np.linalg.norm(X, axis=0)
    X = gram_schmidt(X)
    AX = A @ X
    BX = B @ X
    b_small, lam = lapack_eig(X.T @ AX, X.T @ BX)
    X = X @ b_small
    AX = A @ X
    BX = B @ X
    R = AX - BX * lam[None, :m]
    V = gram_schmidt(np.hstack([X, R]))
    V[:, :m] = V[:, :m] / np.linalg.norm(V[:, :m], axis=0)
    X = V[:, :m].copy()
    R = V[:, m:2 * m].copy()
    AV = A @ V
    BV = B @ V
    b_small, lam = lapack_eig(V.T @ AV, V.T @ BV)
    X = V @ b_small[:, :m]
    AX = A @ X
    BX = B @ X
    R = AX - BX * lam[None, :m]
    OR = np.hstack([np.zeros((n, m)), R])
    P = OR @ b_small[:, :m]
    initial_R = None
    it = 0
    # The loop's n x m and n x 3m arrays live in buffers allocated once: the
    # same arithmetic as allocating them per iteration, without faulting in
    # fresh pages of hundreds of MB every iteration at large n.
    compiled = True
    try:
        from . import lib
        lib()
    except Exception:
        compiled = False
    X, R, P = (np.ascontiguousarray(a, dtype=np.float64) for a in (X, R, P))
    V = np.empty((n, 3 * m))
    AV, BV = np.empty((n, 3 * m)), np.empty((n, 3 * m))
    AX, BX = np.empty((n, m)), np.empty((n, m))
    scratch = np.empty(n * 3 * m) if compiled else None
    for it in range(1, max_itr + 1):
        V[:, :m] = X
        V[:, m:2 * m] = R
        V[:, 2 * m:] = P
        if compiled:
            _gram_schmidt_inplace(V, scratch)
        else:
            V[...] = gram_schmidt(V)
        V[:, :m] /= np.linalg.norm(V[:, :m], axis=0)
        V[:, 2 * m:] /= np.linalg.norm(V[:, 2 * m:], axis=0)
        _mm_into(A, V, AV)
        _mm_into(B, V, BV)
        b_small, lam = lapack_eig(V.T @ AV, V.T @ BV)
        np.matmul(V, b_small[:, :m], out=X)
        _mm_into(A, X, AX)
        _mm_into(B, X, BX)
        np.multiply(BX, lam[None, :m], out=R)
        np.subtract(AX, R, out=R)
        V[:, :m] = 0.0
        np.matmul(V, b_small[:, :m], out=P)
        rmax = max(float(R.max()), -float(R.min()))
        if it == 1:
            initial_R = rmax
        if progress is not None and progress(it, rmax / initial_R, lam[:m], R, BX):
            break  # the caller ended the iteration
        if rmax / initial_R < tol:
            break
    lam = lam[:m].copy()
    if return_iters:
        return lam, X, it
    return lam, X


def dense_generalized_eig(A, B, k: int):
    """Lowest k eigenpairs of the dense pencil (DSPGVD stand-in) for small n."""
    Ad = A.toarray() if hasattr(A, "toarray") else np.asarray(A)
    Bd = B.toarray() if hasattr(B, "toarray") else np.asarray(B)
    w, Z = sla.eigh(Ad, Bd, type=1, subset_by_index=(0, k - 1))
    return w, Z

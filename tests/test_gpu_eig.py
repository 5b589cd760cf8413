"""FEMSolver_%eig (LOBPCG) on the GPU against dense FP64 eigen solves.

The oracle is LAPACK's generalized symmetric-definite solver (scipy's
eigh(A, B, type=1), the DSPGVD stand-in) on the oracle-assembled, reduced
(fix_eig rows/columns removed, reduce_crs_matrix) K and M.  Bars: eigenvalues
within 1e-8 relative (FP64) and 1e-7 (mixed), eigenvectors B-orthonormal to
1e-8 with relative residuals |K x - lambda M x| / (lambda |M x|) <= 1e-7.
"""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

import oracle as O
from plantfem_gb300 import FEMDomain, FEMSolver, problems

pytestmark = pytest.mark.gpu


def cantilever_solver(n):
    p = problems.cantilever(n)
    dom = p["domain"]
    s = FEMSolver()
    s.setDomain(dom)
    s.setCRS(3)
    s.assembleMass(p["rho"])
    s.keepThisMatrixAs("B")
    s.zeros()
    s.assembleStiffness(p["E"], p["nu"])
    s.keepThisMatrixAs("A")
    s.fix_eig(p["fix_ids"])
    s.use_LOBPCG = True
    return s, p


def dense_reference(p, nev):
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    K = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=p["E"], nu=p["nu"])
    M = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "mass", rho=p["rho"])
    rk, ck, vk = O.reduce_crs(rp, ci, K, p["fix_ids"])
    rm, cm, vm = O.reduce_crs(rp, ci, M, p["fix_ids"])
    Kr = O.crs_to_scipy(rk, ck, vk).toarray()
    Mr = O.crs_to_scipy(rm, cm, vm).toarray()
    w = sla.eigh(Kr, Mr, type=1, eigvals_only=True, subset_by_index=(0, nev - 1))
    Kf = O.crs_to_scipy(rp, ci, K)
    Mf = O.crs_to_scipy(rp, ci, M)
    return w, Kf, Mf


@pytest.mark.parametrize("precision,tol_lam", [("fp64", 1e-8), ("mixed", 1e-7)])
def test_eig_cantilever_vs_dense(cuda, precision, tol_lam):
    nev = 6
    s, p = cantilever_solver(5)
    s.LOBPCG_TOL = 1e-9
    lam, X = s.eig(nev, block_size=8, precision=precision)
    assert s.last_info["status"] == 0, s.last_info
    w, Kf, Mf = dense_reference(p, nev)
    assert np.abs(lam - w).max() / np.abs(w).max() <= tol_lam, (lam, w)
    fixed = p["fix_ids"] - 1
    assert np.abs(X[fixed]).max() == 0.0
    G = X.T @ (Mf @ X)
    assert np.abs(G - np.eye(nev)).max() <= 1e-8
    R = Kf @ X - (Mf @ X) * lam[None, :]
    R[fixed] = 0.0
    rel = np.linalg.norm(R, axis=0) / (np.abs(lam) * np.linalg.norm(Mf @ X, axis=0))
    assert rel.max() <= 1e-7, rel


def test_eig_reference_stop_rule(cuda):
    s, p = cantilever_solver(4)
    s.LOBPCG_TOL = 1e-8
    lam, _ = s.eig(4, block_size=8, stop_rule="reference", eigen_vectors=False)
    w, _, _ = dense_reference(p, 4)
    assert np.abs(lam - w).max() / w.max() <= 1e-6


def test_lobpcg_sample_kat_gpu(cuda):
    """Tutorial/std/LOBPCG_sample.f90: n=3000 pencil, m=3, TOL 1e-8; lambda_1 vs
    LAPACK (the tutorial grades < 1e-7 "GOOD", < 1e-14 "EXCELLENT")."""
    n = 3000
    i = np.arange(1, n + 1, dtype=float)
    A = sp.diags([np.full(n - 2, 0.3), np.full(n - 1, 0.5), i, np.full(n - 1, 0.5), np.full(n - 2, 0.3)],
                 [-2, -1, 0, 1, 2], format="lil")
    A[0, 2] += 1.0
    A[2, 0] += 1.0
    A[3, 1] += 1.0
    A[1, 3] += 1.0
    A = A.tocsr()
    B = sp.diags([np.full(n - 1, 0.5), i, np.full(n - 1, 0.5)], [-1, 0, 1], format="csr")
    s = FEMSolver()
    for M, name in ((A, "A"), (B, "B")):
        M = M.tocsr()
        M.sort_indices()
        s.setCRS(CRS=((M.indptr + 1).astype(np.int64), (M.indices + 1).astype(np.int32), M.data))
        s.keepThisMatrixAs(name)
    s.use_LOBPCG = True
    s.LOBPCG_TOL = 1e-10
    lam, X = s.eig(3, block_size=8, preconditioning="Jacobi")
    w = sla.eigh(A.toarray(), B.toarray(), type=1, eigvals_only=True, subset_by_index=(0, 2))
    assert abs(lam[0] - w[0]) < 1e-7
    assert np.abs(lam - w).max() / w.max() < 1e-9


# ----------------------------------------------- the dense branch (the default)
def _check_pairs(lam, X, Kf, Mf, fixed, tol_res=1e-8):
    assert np.abs(X[fixed]).max() == 0.0
    G = X.T @ (Mf @ X)
    assert np.abs(G - np.eye(X.shape[1])).max() <= 1e-9
    R = Kf @ X - (Mf @ X) * lam[None, :]
    R[fixed] = 0.0
    rel = np.linalg.norm(R, axis=0) / (np.abs(lam) * np.linalg.norm(Mf @ X, axis=0))
    assert rel.max() <= tol_res, rel.max()


def test_eig_dense_default_branch_vs_oracle(cuda):
    """use_LOBPCG = .false. (the reference's default): every eigenpair of the
    fix_eig-reduced pencil, ascending, as DSPGVD returns them; against the
    dense LAPACK solve of the oracle-assembled, reduced matrices."""
    s, p = cantilever_solver(4)
    s.use_LOBPCG = False
    lam, X = s.eig()
    nred = 3 * p["domain"].nn() - len(p["fix_ids"])
    assert lam.shape == (nred,) and X.shape == (3 * p["domain"].nn(), nred)
    assert np.all(np.diff(lam) >= 0.0)
    w, Kf, Mf = dense_reference(p, nred)
    assert np.abs(lam - w).max() <= 1e-10 * np.abs(w).max()
    assert np.all(np.abs(lam - w) <= 1e-9 * np.abs(w))
    _check_pairs(lam, X, Kf, Mf, p["fix_ids"] - 1)
    # the lowest num_eigen pairs only
    lam6, X6 = s.eig(6)
    assert lam6.shape == (6,) and np.array_equal(lam6, lam[:6])
    _check_pairs(lam6, X6, Kf, Mf, p["fix_ids"] - 1)


def test_eig_dense_lobpcg_sample_kat(cuda):
    """Tutorial/std/LOBPCG_sample.f90 compares LOBPCG with DSPGVD on the n=3000
    pencil: the dense branch is the DSPGVD side; lambda_1..3 vs LAPACK."""
    n = 3000
    i = np.arange(1, n + 1, dtype=float)
    A = sp.diags([np.full(n - 2, 0.3), np.full(n - 1, 0.5), i, np.full(n - 1, 0.5), np.full(n - 2, 0.3)],
                 [-2, -1, 0, 1, 2], format="lil")
    A[0, 2] += 1.0
    A[2, 0] += 1.0
    A[3, 1] += 1.0
    A[1, 3] += 1.0
    A = A.tocsr()
    B = sp.diags([np.full(n - 1, 0.5), i, np.full(n - 1, 0.5)], [-1, 0, 1], format="csr")
    s = FEMSolver()
    for M, name in ((A, "A"), (B, "B")):
        M = M.tocsr()
        M.sort_indices()
        s.setCRS(CRS=((M.indptr + 1).astype(np.int64), (M.indices + 1).astype(np.int32), M.data))
        s.keepThisMatrixAs(name)
    lam, X = s.eig(3)
    w = sla.eigh(A.toarray(), B.toarray(), type=1, eigvals_only=True, subset_by_index=(0, 2))
    assert abs(lam[0] - w[0]) < 1e-12
    assert np.abs(lam - w).max() / w.max() < 1e-12


def test_eig_dense_refuses_large_problems(cuda):
    """The dense branch stops at 4096 unknowns with PFG_E_UNSUPPORTED (before
    allocating): larger problems take use_LOBPCG."""
    from plantfem_gb300 import _native as N
    s, p = cantilever_solver(12)  # 6,084 reduced unknowns
    s.use_LOBPCG = False
    with pytest.raises(N.NativeError) as e:
        s.eig(5)
    assert e.value.code == -9 and "use_LOBPCG" in str(e.value)

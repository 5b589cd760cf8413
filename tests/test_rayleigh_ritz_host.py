"""The host solver of LOBPCG's Rayleigh-Ritz problems (no GPU needed).

pfg::small_generalized_eig (csrc/lobpcg.cu) returns the lowest k pairs of the
m x m pencil (A, B) that the Gram matrices of [X W P] form each iteration
(SparseClass.f90:2063-2110 hands the same pencil to LAPACK_EIG / DSPGVD).  It
is an internal C++ function of libpfg.so, called here by its symbol.  Checked
against scipy's generalized symmetric-definite solver: eigenvalues, residuals
|A c - lambda B c| and B-orthonormality of the returned coefficients, on
random pencils, pencils with coincident eigenvalues (as the symmetric modes of
a square cantilever give) and badly scaled ones (as LOBPCG's blocks are).
"""
import ctypes
import os

import numpy as np
import pytest
import scipy.linalg as sla

SYMBOL = "_ZN3pfg21small_generalized_eigEiPKdS1_idPdS2_"  # pfg::small_generalized_eig(int, const double*, const double*, int, double, double*, double*)


@pytest.fixture(scope="module")
def rr():
    from plantfem_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from plantfem_gb300.build import build
        build()
    f = getattr(ctypes.CDLL(_native.LIB_PATH), SYMBOL)
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                  ctypes.c_void_p]

    def run(A, B, k, rank_tol=1e-13):
        m = A.shape[0]
        lam = np.zeros(k)
        C = np.zeros((k, m))
        Af, Bf = np.asfortranarray(A), np.asfortranarray(B)
        got = f(m, Af.ctypes.data, Bf.ctypes.data, k, rank_tol, lam.ctypes.data, C.ctypes.data)
        return got, lam, C.T

    return run


def _pencil(kind, rng, m):
    if kind == "random":
        A = rng.standard_normal((m, m))
        G = rng.standard_normal((m, m))
        return A + A.T, G @ G.T + m * np.eye(m)
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    if kind == "coincident":
        ev = np.sort(rng.uniform(1.0, 100.0, m))
        ev[1] = ev[0]
        if m > 10:
            ev[3] = ev[2]
            ev[4] = ev[5] = ev[6]
            ev[10] = ev[9] * (1 + 1e-15)
        G = 0.1 * rng.standard_normal((m, m))
        B = G @ G.T + np.eye(m)
        L = np.linalg.cholesky(B)
        return L @ (Q @ np.diag(ev) @ Q.T) @ L.T, B
    ev = np.sort(rng.uniform(1.0, 1e4, m))  # "graded": rows and columns scaled over 7 decades
    s = np.exp(rng.uniform(-8.0, 8.0, m))
    return (Q @ np.diag(ev) @ Q.T) * np.outer(s, s), np.diag(s * s)


@pytest.mark.parametrize("kind", ["random", "coincident", "graded"])
@pytest.mark.parametrize("m,k", [(72, 24), (48, 16), (9, 3), (3, 1)])
def test_lowest_pairs_match_scipy(rr, kind, m, k):
    rng = np.random.default_rng(m * 7 + k)
    for _ in range(20):
        A, B = _pencil(kind, rng, m)
        got, lam, C = rr(A, B, k)
        assert got == k
        w = sla.eigh(A, B, eigvals_only=True)[:k]
        assert np.abs(lam - w).max() <= 1e-13 * np.abs(w).max()
        R = A @ C - (B @ C) * lam[None, :]
        res = np.linalg.norm(R, axis=0) / (np.linalg.norm(A, 2) * np.linalg.norm(C, axis=0))
        assert res.max() <= 1e-13
        assert np.abs(C.T @ B @ C - np.eye(k)).max() <= 1e-12


def test_rank_deficient_basis_is_truncated(rr):
    """B singular (a dependent direction in [X W P]): the solver drops it and
    still returns B-orthonormal pairs of the remaining pencil."""
    rng = np.random.default_rng(3)
    m, k = 12, 4
    V = rng.standard_normal((40, m))
    V[:, -1] = V[:, 0] + V[:, 1]  # dependent column
    K = rng.standard_normal((40, 40))
    K = K @ K.T + 40 * np.eye(40)
    A, B = V.T @ K @ V, V.T @ V
    got, lam, C = rr(A, B, k)
    assert got == k
    Vr = V[:, :-1]
    w = sla.eigh(Vr.T @ K @ Vr, Vr.T @ Vr, eigvals_only=True)[:k]
    assert np.abs(lam - w).max() <= 1e-10 * np.abs(w).max()
    assert np.abs(C.T @ B @ C - np.eye(k)).max() <= 1e-9

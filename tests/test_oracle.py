"""Pinning the CPU oracle (no GPU needed).

The oracle is only trusted after it reproduces what the reference itself
says: its own C SpMV (compiled from the reference source into oracle/_ref),
the equality of its two pattern builders (Tutorial/fem/CRS_Zero_Matrix.f90),
the gravity-bar stress (Tutorial/fem/benchmark_bar_in_gravity_field.f90:63-67),
the LOBPCG sample (Tutorial/std/LOBPCG_sample.f90) and the 1-D Poisson solve
(Tutorial/fem/FEMSolver_PoissonMatrix.f90), plus analytic known answers.
"""
import hashlib
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
from oracle import lobpcg as L

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_golden_manifest_hashes():
    man = json.load(open(os.path.join(GOLD, "MANIFEST.json")))
    for name, h in man["files"].items():
        assert hashlib.sha256(open(os.path.join(GOLD, name), "rb").read()).hexdigest() == h


def test_oracle_reproduces_goldens():
    g = np.load(os.path.join(GOLD, "hex8_elements.npz"))
    for i in range(3):
        np.testing.assert_array_equal(O.hex8_stiffness(g["xe"][i], 1.0e4, 0.3), g["Ke"][i])
        np.testing.assert_array_equal(O.hex8_mass(g["xe"][i], 1.0e3), g["Me"][i])
    p = np.load(os.path.join(GOLD, "patterns.npz"))
    for key in ("111", "222", "321"):
        nx, ny, nz = (int(c) for c in key)
        xyz, en = O.cube3d(nx, ny, nz)
        rp, ci = O.zero_matrix(xyz.shape[0], en, 3)
        np.testing.assert_array_equal(rp, p["rp_" + key])
        np.testing.assert_array_equal(ci, p["ci_" + key])


def _random_crs(n, density, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=seed, format="csr") + sp.eye(n, format="csr")
    rp = (A.indptr + 1).astype(np.int64)
    ci = (A.indices + 1).astype(np.int32)
    return rp, ci, A.data.astype(np.float64), rng.standard_normal(n)


@pytest.mark.skipif(O.ref_lib() is None, reason="reference C SpMV not compiled here (no reference checkout)")
def test_spmv_bit_exact_vs_reference_c():
    """orc_crs_spmv_real64 == the reference's crs_spmv_real64 (SparseClass-c.c:53-65), bit for bit."""
    R = O.ref_lib()
    for seed, n in ((0, 1), (1, 37), (2, 1000)):
        rp, ci, val, x = _random_crs(n, 0.05, seed)
        y0 = np.random.default_rng(seed + 9).standard_normal(n)
        y_ref = y0.copy()
        R.crs_spmv_real64(val, rp, ci, x, y_ref, n, ci.shape[0])
        y_orc = y0.copy()
        O.crs_spmv_real64(val, rp, ci, x, y_orc)
        np.testing.assert_array_equal(y_orc, y_ref)
    # the FEM matrix of a small cube, too
    xyz, en = O.cube3d(3, 3, 3)
    rp, ci = O.zero_matrix(xyz.shape[0], en, 3)
    val = O.assemble(xyz, en, rp, ci, "stiffness", E=1.0e4, nu=0.3)
    x = np.random.default_rng(3).standard_normal(rp.shape[0] - 1)
    y_ref = np.zeros_like(x)
    R.crs_spmv_real64(val, rp, ci, x, y_ref, x.shape[0], ci.shape[0])
    np.testing.assert_array_equal(O.spmv(rp, ci, val, x), y_ref)


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 2, 2), (3, 2, 1), (5, 4, 3), (10, 10, 20)])
def test_pattern_ell_equals_legacy_coo(shape):
    """Tutorial/fem/CRS_Zero_Matrix.f90:22-29: both builders give the same arrays."""
    xyz, en = O.cube3d(*shape)
    a = O.zero_matrix(xyz.shape[0], en, 3)
    b = O.zero_matrix(xyz.shape[0], en, 3, legacy=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    # structured grid: sum over nodes of node neighbours = prod(3 n_axis + 1)
    nodes_nb = np.prod([3 * s + 1 for s in shape])
    assert a[0][-1] - 1 == 9 * nodes_nb


def _gravity_bar(deformed):
    xyz, en = O.cube3d(10, 10, 100)
    xyz[:, 2] *= 10.0 / (xyz[:, 2].max() - xyz[:, 2].min())
    nn = xyz.shape[0]
    rp, ci = O.zero_matrix(nn, en, 3)
    val = O.assemble(xyz, en, rp, ci, "stiffness", E=2.17e7, nu=0.0)
    rhs = O.body_force(xyz, en, 2.4, [0, 0, -9.8])
    bot = np.nonzero(xyz[:, 2] <= xyz[:, 2].min())[0]
    fixed = np.zeros(3 * nn, np.uint8)
    for d in range(3):
        fixed[3 * bot + d] = 1
    O.apply_fix(rp, ci, val, rhs, fixed, np.zeros(3 * nn))
    x, rc, it = O.bicgstab_crs2(rp, ci, val, rhs)
    assert rc == 0
    if deformed:
        xyz = xyz + x.reshape(nn, 3)
    S = O.element_stress(xyz, en, x, 2.17e7, 0.0)
    return np.trace(S[0])


@pytest.mark.slow
def test_gravity_bar_kat():
    """benchmark_bar_in_gravity_field.f90:63-67: bottom-element I1 stress is
    -234.026 after cube%deform (simulated) and -234.024 in theory."""
    assert abs(_gravity_bar(deformed=True) - (-234.026)) < 1e-3
    assert abs(_gravity_bar(deformed=False) - (-234.024)) < 1e-3


def test_lobpcg_sample_kat():
    """Tutorial/std/LOBPCG_sample.f90: n=3000 pentadiagonal/tridiagonal pencil,
    m=3, TOL=1e-8; lambda_1 against LAPACK's DSPGVD, graded good if < 1e-7."""
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
    lam, X, it = L.lobpcg_crs(A, B, m=3, max_itr=2000, tol=1e-8, seed=1, return_iters=True)
    w, _ = L.dense_generalized_eig(A, B, 3)
    assert abs(lam[0] - w[0]) < 1e-7


def test_gram_schmidt_compiled_equals_numpy_loop():
    """GramSchmidt (SparseClass.f90:2243-2275): the compiled restatement
    (orc_gram_schmidt, both memory orders) equals the numpy loop, skips a zero
    column and returns orthonormal columns."""
    rng = np.random.default_rng(11)
    V = rng.random((3000, 20))
    V[:, 5] = 0.0
    ref = L.gram_schmidt_numpy(V)
    for W in (V, np.asfortranarray(V)):
        got = L.gram_schmidt(W)
        assert np.abs(got - ref).max() <= 1e-13
    keep = [j for j in range(20) if j != 5]
    Q = ref[:, keep]
    assert np.abs(Q.T @ Q - np.eye(19)).max() <= 1e-12
    assert np.all(ref[:, 5] == 0.0)


def test_poisson_1d_kat():
    """Tutorial/fem/FEMSolver_PoissonMatrix.f90:18-45 through setCRS(CRS)+solve."""
    n = 100
    A = np.zeros((n, n))
    for r in range(n):
        for c in (r - 1, r, r + 1):
            if 0 <= c < n:
                A[r, c] = 2.0 if c == r else -1.0
    A[:, 0] = 0.0
    A[0, :] = 0.0
    A[0, 0] = 1.0
    S = sp.csr_matrix(A)
    # COO%update keeps explicit zeros in the pattern; the values are what matter here
    rp = (S.indptr + 1).astype(np.int64)
    ci = (S.indices + 1).astype(np.int32)
    rhs = np.zeros(n)
    rhs[0] = rhs[1] = 10.0
    x, rc, it = O.bicgstab_crs2(rp, ci, S.data.copy(), rhs, relative_er=1e-5)
    assert rc == 0
    exact = np.linalg.solve(A, rhs)
    assert np.abs(x - exact).max() / np.abs(exact).max() < 1e-3


def test_element_matrix_properties():
    """Symmetry, six rigid-body modes of Ke, total mass of Me, patch test."""
    g = np.load(os.path.join(GOLD, "hex8_elements.npz"))
    for i in range(3):
        Ke, Me, xe = g["Ke"][i], g["Me"][i], g["xe"][i]
        np.testing.assert_allclose(Ke, Ke.T, rtol=0, atol=1e-9 * np.abs(Ke).max())
        w = np.linalg.eigvalsh(0.5 * (Ke + Ke.T))
        assert np.sum(np.abs(w) < 1e-8 * w.max()) == 6 if i < 2 else True
        for d in range(3):  # rigid translation gives zero force
            u = np.zeros(24)
            u[d::3] = 1.0
            assert np.abs(Ke @ u).max() < 1e-9 * np.abs(Ke).max()
        vol = abs(np.linalg.det(np.stack([xe[1] - xe[0], xe[3] - xe[0], xe[4] - xe[0]])))
        if i < 2:
            assert abs(Me.sum() - 3 * 1.0e3 * vol) < 1e-9 * Me.sum()
    # uniaxial patch test, nu = 0: linear displacement is reproduced exactly
    xe = g["xe"][1]
    Ke = O.hex8_stiffness(xe, 1.0, 0.0)
    u = np.zeros(24)
    u[2::3] = 0.01 * xe[:, 2]
    f = Ke @ u
    # nodal forces only in z, equal and opposite on the two z faces
    assert np.abs(f[0::3]).max() < 1e-14 and np.abs(f[1::3]).max() < 1e-14
    area = 0.5 * 0.25
    assert abs(f[2::3][xe[:, 2] > 0].sum() - 0.01 * area) < 1e-14


def test_bc_elimination_and_reduce():
    g = np.load(os.path.join(GOLD, "cube4_lognormal.npz"))
    val, rhs = g["val_assembled"].copy(), g["rhs_in"].copy()
    O.apply_fix(g["rp"], g["ci"], val, rhs, g["fixed"], np.zeros(rhs.shape[0]))
    np.testing.assert_array_equal(val, g["val_eliminated"])
    np.testing.assert_array_equal(rhs, g["rhs_eliminated"])
    K = O.crs_to_scipy(g["rp"], g["ci"], val)
    assert abs(K - K.T).max() < 1e-9 * abs(K).max()
    ids = np.nonzero(g["fixed"])[0] + 1
    rp, ci, v = O.reduce_crs(g["rp"], g["ci"], g["val_assembled"], np.concatenate([ids[::-1], ids[:3]]))
    R = O.crs_to_scipy(rp, ci, v)
    keep = np.nonzero(g["fixed"] == 0)[0]
    F = O.crs_to_scipy(g["rp"], g["ci"], g["val_assembled"])
    assert abs(R - F[keep][:, keep]).max() == 0.0


def test_oracle_bicgstab_matches_pcg():
    g = np.load(os.path.join(GOLD, "cube4_lognormal.npz"))
    x, rc, it = O.bicgstab_crs2(g["rp"], g["ci"], g["val_eliminated"], g["rhs_eliminated"], relative_er=1e-12,
                                er0=1e-30)
    assert rc == 0
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) < 1e-9


def _dense_crs(A):
    """Dense matrix -> 1-based CRS with every entry stored, columns sorted."""
    n = A.shape[0]
    rp = np.arange(0, n * n + 1, n, dtype=np.int64) + 1
    ci = np.tile(np.arange(1, n + 1, dtype=np.int32), n)
    return rp, ci, np.ascontiguousarray(A, dtype=np.float64).ravel()


@pytest.mark.parametrize("sorted_", [False, True])
def test_ilu0_tutorial_kats(sorted_):
    """Tutorial/std/ILU_test.f90: the 4x4 factor listed in its comments
    (:33-37) and the 3x3 factor it checks entry by entry (:125-178)."""
    A4 = np.array([[1, 1, 0, 3], [2, 1, -1, 1], [3, -1, -1, 2], [-1, 2, 3, -1]], float)
    F4 = np.array([[1, 1, 0, 3], [2, -1, -1, -5], [3, 4, 3, 13], [-1, -3, 0, -13]], float)
    rp, ci, v = _dense_crs(A4)
    assert np.array_equal(O.ilu0(rp, ci, v, sorted_).reshape(4, 4), F4)
    A3 = np.array([[5, 6, 7], [10, 20, 23], [15, 50, 67]], float)
    F3 = np.array([[5, 6, 7], [2, 8, 9], [3, 4, 10]], float)
    rp, ci, v = _dense_crs(A3)
    assert np.array_equal(O.ilu0(rp, ci, v, sorted_).reshape(3, 3), F3)


def test_ilu_rhs_solve_tutorial_kat():
    """Tutorial/std/CRS_test.f90:90-94: ILU(0, RHS=[2, 3, 4]) of the 3x3 matrix
    gives [0.54, -0.35, 0.20]; on a dense pattern ILU(0) is the LU factor, so
    the ILU solve is exact for any right-hand side."""
    A = np.array([[5, 6, 7], [10, 20, 23], [15, 50, 67]], float)
    rp, ci, v = _dense_crs(A)
    lu = O.ilu0(rp, ci, v)
    np.testing.assert_allclose(O.ilu_solve(rp, ci, lu, [2.0, 3.0, 4.0]), [0.54, -0.35, 0.20], rtol=0, atol=1e-14)
    rng = np.random.default_rng(6)
    B = rng.standard_normal((7, 7)) + 7 * np.eye(7)
    rp, ci, v = _dense_crs(B)
    b = rng.standard_normal(7)
    np.testing.assert_allclose(O.ilu_solve(rp, ci, O.ilu0(rp, ci, v), b), np.linalg.solve(B, b), rtol=1e-12)


def test_pbicgstab_ilu_tutorial_kat():
    """Tutorial/std/PBiCGSTAB_ILU.f90: x = [0.54, -0.35, 0.20] for the 3x3
    system, er = relative_er = 1e-13."""
    rp, ci, v = _dense_crs(np.array([[5, 6, 7], [10, 20, 23], [15, 50, 67]], float))
    x, rc, it = O.bicgstab_ilu(rp, ci, v, np.array([2.0, 3.0, 4.0]), er0=1e-13, relative_er=1e-13)
    assert rc == 0 and it <= 6
    np.testing.assert_allclose(x, [0.54, -0.35, 0.20], rtol=0, atol=1e-12)


def _shuffled_rows(rp, ci, v, seed):
    """The same matrix with each row's entries stored in a random order."""
    rng = np.random.default_rng(seed)
    ci2, v2 = ci.copy(), v.copy()
    for i in range(rp.shape[0] - 1):
        s, e = rp[i] - 1, rp[i + 1] - 1
        p = s + rng.permutation(e - s)
        ci2[s:e], v2[s:e] = ci[p], v[p]
    return ci2, v2


def test_ilu0_defining_property_and_orders():
    """Sorted order: (L U)_ij = a_ij on the pattern (the ILU(0) identity), the
    stored order equals it when the rows are sorted, and D^-1 L^-1 inverts
    L D.  With rows stored out of order the stored-order factor differs, as
    in the reference."""
    rng = np.random.default_rng(4)
    n = 60
    A = sp.random(n, n, density=0.12, random_state=5, format="csr") + sp.diags(np.full(n, 6.0))
    A = (A + A.T).tocsr()
    A.sort_indices()
    rp = (A.indptr + 1).astype(np.int64)
    ci = (A.indices + 1).astype(np.int32)
    v = A.data.copy()
    lu = O.ilu0(rp, ci, v, sorted=True)
    assert np.array_equal(lu, O.ilu0(rp, ci, v, sorted=False))
    F = sp.csr_matrix((lu, ci - 1, rp - 1), shape=(n, n)).toarray()
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    mask = A.toarray() != 0
    np.testing.assert_allclose((L @ U)[mask], A.toarray()[mask], rtol=0, atol=1e-12 * abs(A).max())
    w = rng.standard_normal(n)
    out = O.ilu_apply(rp, ci, lu, w)
    np.testing.assert_allclose(L @ (np.diag(np.diag(U)) @ out), w, rtol=0, atol=1e-12 * abs(w).max())
    ci2, v2 = _shuffled_rows(rp, ci, v, 1)
    lu_sorted = O.ilu0(rp, ci2, v2, sorted=True)
    back = sp.csr_matrix((lu_sorted, ci2 - 1, rp - 1), shape=(n, n)).toarray()
    np.testing.assert_allclose(back, F, rtol=0, atol=1e-14 * abs(F).max())
    lu_stored = O.ilu0(rp, ci2, v2, sorted=False)
    assert not np.allclose(sp.csr_matrix((lu_stored, ci2 - 1, rp - 1), shape=(n, n)).toarray(), F)


def test_bicgstab_ilu_fem_orders():
    """On an eliminated hex8 stiffness matrix (first-appearance column order)
    the sorted-order factor makes bicgstab_CRS_ILU converge in fewer
    iterations than bicgstab_CRS_2 needs; the stored-order factor, which is
    what the reference computes for these rows, carries unscaled updates
    into L and its preconditioned solve does not converge."""
    nx = 4
    nodcoord, elemnod = O.cube3d(nx, nx, nx)
    nn = nodcoord.shape[0]
    rp, ci = O.zero_matrix(nn, elemnod, 3)
    val = O.assemble(nodcoord, elemnod, rp, ci, "stiffness", E=np.full(nx ** 3, 1e4), nu=np.full(nx ** 3, 0.3))
    b = np.zeros(3 * nn)
    top = np.where(np.isclose(nodcoord[:, 2], 1.0))[0]
    b[3 * top + 2] = -1.0 / top.shape[0]
    fixed = np.zeros(3 * nn, np.uint8)
    bot = np.where(np.isclose(nodcoord[:, 2], 0.0))[0]
    for d in range(3):
        fixed[3 * bot + d] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * nn))
    x_ref = sp.linalg.spsolve(O.crs_to_scipy(rp, ci, val).tocsc(), b)
    x, rc, it = O.bicgstab_ilu(rp, ci, val, b, sorted=True, er0=1e-30, relative_er=1e-12)
    assert rc == 0
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    _, rc2, it2 = O.bicgstab_crs2(rp, ci, val, b, er0=1e-30, relative_er=1e-12)
    assert rc2 == 0 and it < it2
    lu_st = O.ilu0(rp, ci, val, sorted=False)
    assert np.abs(np.tril(O.crs_to_scipy(rp, ci, lu_st).toarray(), -1)).max() > 10.0
    with np.errstate(all="ignore"):
        xs, rcs, _ = O.bicgstab_ilu(rp, ci, val, b, lu=lu_st, er0=1e-30, relative_er=1e-12, itrmax=200)
    assert rcs != 0 or not np.all(np.isfinite(xs)) or np.linalg.norm(xs - x_ref) > 1e-3 * np.linalg.norm(x_ref)

"""ILU(0)-preconditioned BiCGSTAB (preconditioning="ILU") on the GPU.

The factor (ILUCRS, SparseClass.f90:1629-1792) is compared with the oracle's
restatement bit for bit: both take every update as a + (-(l * a_kj)) rounded
twice, in the same order.  The sweep D^-1 L^-1 v (ILU_matvecCRS as it executes,
SparseClass.f90:1795-1852) sums in another order: 1e-12 relative.  Solves
(bicgstab_CRS_ILU, LinearSolverClass.f90:4104-4230) are compared with the
oracle's solve and an FP64 direct solve at 1e-8 relative displacement error.
The tutorial known answers (Tutorial/std/ILU_test.f90, PBiCGSTAB_ILU.f90) run
through the C ABI.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import oracle as O
from plantfem_gb300 import FEMSolver, problems
from plantfem_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _fem(n=5, seed=11):
    p = problems.lognormal(n, seed=seed)
    s = FEMSolver()
    s.setDomain(p["domain"])
    s.setCRS(3)
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    return s, p


def _oracle_system(p):
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=p["E"], nu=p["nu"])
    b = p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    return rp, ci, val, b


def _scalar_matrix(n=50, seed=3):
    A = sp.random(n, n, density=0.15, random_state=seed, format="csr")
    A = (A + A.T + sp.diags(np.full(n, 8.0))).tocsr()
    A.sort_indices()
    return (A.indptr + 1).astype(np.int64), (A.indices + 1).astype(np.int32), A.data.copy()


def _dense_crs(A):
    n = A.shape[0]
    rp = np.arange(0, n * n + 1, n, dtype=np.int64) + 1
    ci = np.tile(np.arange(1, n + 1, dtype=np.int32), n)
    return rp, ci, np.ascontiguousarray(A, dtype=np.float64).ravel()


@pytest.mark.parametrize("sorted_", [False, True])
def test_ilu_factor_bit_exact_fem(cuda, sorted_):
    s, p = _fem()
    s.eliminate()
    lu = s.ILU(sorted=sorted_)
    rp, ci, val, _ = _oracle_system(p)
    grp, gci, gval = s.getCRS()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
    assert np.abs(gval - val).max() <= 1e-12 * np.abs(val).max()  # assembly sums in another order
    # the factorization itself from the same input values
    ref = O.ilu0(rp, ci, gval, sorted=sorted_)
    assert np.array_equal(np.isnan(lu), np.isnan(ref))
    fin = np.isfinite(ref)
    assert np.array_equal(lu[fin], ref[fin])


@pytest.mark.parametrize("sorted_", [False, True])
def test_ilu_factor_bit_exact_scalar(cuda, sorted_):
    rp, ci, v = _scalar_matrix()
    # rows stored out of order, so the two orders differ
    rng = np.random.default_rng(0)
    for i in range(rp.shape[0] - 1):
        a, b = rp[i] - 1, rp[i + 1] - 1
        q = a + rng.permutation(b - a)
        ci[a:b], v[a:b] = ci[q].copy(), v[q].copy()
    s = FEMSolver()
    s.setCRS(CRS=(rp, ci, v))
    lu = s.ILU(sorted=sorted_)
    assert np.array_equal(lu, O.ilu0(rp, ci, v, sorted=sorted_))


def test_ilu_tutorial_kats_gpu(cuda):
    """ILU_test.f90 (3x3 factor checked entry by entry, 4x4 factor in its
    comments) and PBiCGSTAB_ILU.f90 (x = [0.54, -0.35, 0.20])."""
    A3 = np.array([[5, 6, 7], [10, 20, 23], [15, 50, 67]], float)
    s = FEMSolver()
    s.setCRS(CRS=_dense_crs(A3))
    assert np.array_equal(s.ILU().reshape(3, 3), np.array([[5, 6, 7], [2, 8, 9], [3, 4, 10]], float))
    s.setRHS(np.array([2.0, 3.0, 4.0]))
    s.er0 = 1e-13
    s.relative_er = 1e-13
    x = s.solve(preconditioning="ILU")
    np.testing.assert_allclose(x, [0.54, -0.35, 0.20], rtol=0, atol=1e-12)
    A4 = np.array([[1, 1, 0, 3], [2, 1, -1, 1], [3, -1, -1, 2], [-1, 2, 3, -1]], float)
    t = FEMSolver()
    t.setCRS(CRS=_dense_crs(A4))
    F4 = np.array([[1, 1, 0, 3], [2, -1, -1, -5], [3, 4, 3, 13], [-1, -3, 0, -13]], float)
    assert np.array_equal(t.ILU().reshape(4, 4), F4)


def test_ilu_apply_matches_oracle(cuda):
    for sys_ in ("fem", "scalar"):
        if sys_ == "fem":
            s, p = _fem(4)
            s.eliminate()
            rp, ci, val, _ = _oracle_system(p)
        else:
            rp, ci, val = _scalar_matrix(70, 9)
            s = FEMSolver()
            s.setCRS(CRS=(rp, ci, val))
        lu = s.ILU(sorted=True)
        v = np.random.default_rng(1).standard_normal(rp.shape[0] - 1)
        out = s.ILU_matvec(v)
        ref = O.ilu_apply(rp, ci, lu, v)
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max(), sys_


@pytest.mark.parametrize("stop_rule", ["reference", "true_relative"])
def test_ilu_bicgstab_matches_oracle(cuda, stop_rule):
    s, p = _fem(6)
    s.relative_er = 1e-10
    s.er0 = 1e-30
    x = s.solve(preconditioning="ILU", ilu_order="sorted", stop_rule=stop_rule)
    info = s.last_info
    assert info["status"] == 0
    rp, ci, val, b = _oracle_system(p)
    x_direct = sla.spsolve(O.crs_to_scipy(rp, ci, val).tocsc(), b)
    xo, rc, it = O.bicgstab_ilu(rp, ci, val, b, sorted=True, er0=1e-30, relative_er=1e-10)
    assert rc == 0
    if stop_rule == "reference":
        assert abs(info["iterations"] - it) <= 2, (info["iterations"], it)
        np.testing.assert_allclose(x, xo, rtol=0, atol=1e-7 * np.abs(xo).max())
    else:
        assert info["rel_residual"] <= 1e-10
        assert np.linalg.norm(x - x_direct) <= 1e-8 * np.linalg.norm(x_direct)
    # the factor is preconditioning: fewer iterations than unpreconditioned BiCGSTAB
    _, _, it_plain = O.bicgstab_crs2(rp, ci, val, b, er0=1e-30, relative_er=1e-10)
    assert info["iterations"] < it_plain


def test_ilu_factor_kept_until_reset(cuda):
    """FEMSolver_ keeps ILU_MATRIX after its first ILU solve, even when the
    matrix changes (LinearSolverClass.f90:4126-4135); resetILU drops it."""
    s, p = _fem(4)
    s.solve(preconditioning="ILU", ilu_order="sorted", stop_rule="true_relative")
    lu0 = s.ILU(sorted=True)
    s.assembleStiffness(2.0 * p["E"], p["nu"])  # new values, same pattern
    assert np.array_equal(s.ILU(sorted=True), lu0)
    s.resetILU()
    lu1 = s.ILU(sorted=True)
    assert not np.array_equal(lu1, lu0)


def test_ilu_stored_order_on_fem_rows(cuda):
    """With first-appearance column order the stored-order factor carries
    unscaled updates into L; the preconditioned solve then fails or does
    not converge, as the reference's does.  It must end with a status, within
    itrmax, on the GPU as in the oracle."""
    s, p = _fem(4)
    s.itrmax = 200
    s.relative_er = 1e-12
    s.er0 = 1e-30
    rp, ci, val, b = _oracle_system(p)
    with np.errstate(all="ignore"):
        xo, rc, _ = O.bicgstab_ilu(rp, ci, val, b, sorted=False, er0=1e-30, relative_er=1e-12, itrmax=200)
    x_direct = sla.spsolve(O.crs_to_scipy(rp, ci, val).tocsc(), b)
    oracle_failed = rc != 0 or not np.all(np.isfinite(xo)) or \
        np.linalg.norm(xo - x_direct) > 1e-3 * np.linalg.norm(x_direct)
    assert oracle_failed
    try:
        x = s.solve(preconditioning="ILU", ilu_order="stored")
        info = s.last_info
        failed = info["status"] != 0 or not np.all(np.isfinite(x)) or \
            np.linalg.norm(x - x_direct) > 1e-3 * np.linalg.norm(x_direct)
    except N.NativeError:
        failed = True
    assert failed


def test_ilu_apply_uses_the_held_factor(cuda):
    """ILU_matvec applies the factor the solver keeps, whichever order it was
    taken in (it does not refactor)."""
    rp, ci, v = _scalar_matrix(40, 5)
    rng = np.random.default_rng(2)
    for i in range(rp.shape[0] - 1):
        a, b = rp[i] - 1, rp[i + 1] - 1
        q = a + rng.permutation(b - a)
        ci[a:b], v[a:b] = ci[q].copy(), v[q].copy()
    s = FEMSolver()
    s.setCRS(CRS=(rp, ci, v))
    lu = s.ILU(sorted=False)
    w = rng.standard_normal(rp.shape[0] - 1)
    out = s.ILU_matvec(w)
    ref = O.ilu_apply(rp, ci, lu, w)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.array_equal(s.ILU(sorted=False), lu)


def test_ilu_rhs_solve(cuda):
    """CRS_%ILU(0, RHS) (Tutorial/std/CRS_test.f90:90-94: [0.54, -0.35, 0.20]),
    a dense system (ILU(0) = LU: exact), and an FEM system against the oracle's
    restatement with the same factor."""
    s = FEMSolver()
    s.setCRS(CRS=_dense_crs(np.array([[5, 6, 7], [10, 20, 23], [15, 50, 67]], float)))
    np.testing.assert_allclose(s.ILU(RHS=[2.0, 3.0, 4.0]), [0.54, -0.35, 0.20], rtol=0, atol=1e-13)
    rng = np.random.default_rng(8)
    B = rng.standard_normal((10, 10)) + 10 * np.eye(10)
    t = FEMSolver()
    t.setCRS(CRS=_dense_crs(B))
    b = rng.standard_normal(10)
    np.testing.assert_allclose(t.ILU(RHS=b), np.linalg.solve(B, b), rtol=1e-11)
    for sys_ in ("fem", "scalar"):
        if sys_ == "fem":
            u, p = _fem(4)
            u.eliminate()
            rp, ci, _, _ = _oracle_system(p)
        else:
            rp, ci, val = _scalar_matrix(60, 11)
            u = FEMSolver()
            u.setCRS(CRS=(rp, ci, val))
        lu = u.ILU(sorted=True)
        r = rng.standard_normal(rp.shape[0] - 1)
        x = u.ILU(sorted=True, RHS=r)
        ref = O.ilu_solve(rp, ci, lu, r)
        assert np.abs(x - ref).max() <= 1e-11 * np.abs(ref).max(), sys_


def test_ilu_refuses_cg_and_mixed(cuda):
    s, p = _fem(3)
    s.eliminate()
    import ctypes as C
    lib = N.load()
    for alg, prec in ((N.ALG_CG, N.PREC_FP64), (N.ALG_BICGSTAB, N.PREC_MIXED)):
        o = N.default_opts(algorithm=alg, precision=prec, precond=N.PC_ILU0_SORTED)
        x = np.zeros(s.ndof())
        rc = lib.pfg_solve(s._h, C.byref(o), None, N.ptr(x), None)
        assert rc == -9  # PFG_E_UNSUPPORTED

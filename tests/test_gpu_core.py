"""Parity of the GPU path with the CPU oracle: pattern, assembly, Dirichlet
elimination, SpMV and the Krylov solves, all through the C ABI.

Tolerances: index arrays are compared bit for bit; the elimination is bit for
bit given the same assembled values; assembled values within 1e-12 of the
largest entry (different summation order of element contributions); SpMV
within 1e-13 relative (warp-tree vs serial row sums); solutions within 1e-8
relative to the FP64 oracle solved to 1e-12 (the accuracy bar of the path).
"""
import os

import numpy as np
import pytest

import oracle as O
from plantfem_gb300 import FEMDomain, FEMSolver, _native, crs_spmv_real32, crs_spmv_real64, linear_solver_crs
from plantfem_gb300 import problems

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def solver_for(dom):
    s = FEMSolver()
    s.setDomain(dom)
    s.setCRS(3)
    return s


def oracle_system(dom, E, nu, rhs, fix_ids):
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=E, nu=nu)
    b = rhs.copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[fix_ids - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    return rp, ci, val, b


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 2, 2), (3, 2, 1), (7, 5, 3), (20, 20, 20)])
def test_pattern_bit_exact(cuda, shape):
    dom = FEMDomain().create("Cube3D", *shape)
    s = solver_for(dom)
    rp, ci, val = s.getCRS()
    orp, oci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert not val.any()


def test_pattern_goldens(cuda):
    g = np.load(os.path.join(GOLD, "patterns.npz"))
    for key in ("111", "222", "321"):
        dom = FEMDomain().create("Cube3D", *(int(c) for c in key))
        rp, ci, _ = solver_for(dom).getCRS()
        np.testing.assert_array_equal(rp, g["rp_" + key])
        np.testing.assert_array_equal(ci, g["ci_" + key])


def _skewed(shape, seed=0):
    dom = FEMDomain().create("Cube3D", *shape)
    rng = np.random.default_rng(seed)
    h = 1.0 / max(shape)
    dom.nodcoord = dom.nodcoord + rng.uniform(-0.15 * h, 0.15 * h, size=dom.nodcoord.shape)
    return dom


@pytest.mark.parametrize("skew", [False, True])
def test_stiffness_assembly_vs_oracle(cuda, skew):
    shape = (5, 4, 3)
    dom = _skewed(shape) if skew else FEMDomain().create("Cube3D", *shape)
    rng = np.random.default_rng(1)
    E = np.exp(rng.normal(np.log(1e4), 0.5, dom.ne()))
    nu = rng.uniform(0.1, 0.45, dom.ne())
    s = solver_for(dom)
    s.assembleStiffness(E, nu)
    _, _, val = s.getCRS()
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    ref = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=E, nu=nu)
    assert np.abs(val - ref).max() <= 1e-12 * np.abs(ref).max()


def test_assembly_is_deterministic(cuda):
    dom = FEMDomain().create("Cube3D", 9, 8, 7)
    E = problems.lognormal_E(dom.ne(), seed=3)
    a = solver_for(dom)
    a.assembleStiffness(E, 0.3)
    b = solver_for(dom)
    b.assembleStiffness(E, 0.3)
    np.testing.assert_array_equal(a.getCRS()[2], b.getCRS()[2])


@pytest.mark.parametrize("lumped", [False, True])
def test_mass_assembly_vs_oracle(cuda, lumped):
    dom = _skewed((4, 3, 3), seed=2)
    rho = np.random.default_rng(4).uniform(500, 1500, dom.ne())
    s = solver_for(dom)
    s.assembleMass(rho, Lumped=lumped)
    _, _, val = s.getCRS()
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    ref = np.zeros(ci.shape[0])
    en = np.asfortranarray(dom.elemnod).T.reshape(-1).copy()
    for e in range(dom.ne()):
        Me = O.hex8_mass(dom.element_coords(e + 1), rho[e], lumped=lumped)
        assert O.lib().orc_set_matrix(rp, ci, ref, dom.ne(), en, e, 3, np.ascontiguousarray(Me.T).reshape(-1)) == 0
    assert np.abs(val - ref).max() <= 1e-12 * np.abs(ref).max()


def test_set_matrix_and_vector_paths(cuda):
    dom = FEMDomain().create("Cube3D", 3, 3, 2)
    Ke = O.element_stiffness_all(dom.nodcoord, dom.elemnod, 1e4, 0.3)
    s = solver_for(dom)
    for e in range(dom.ne()):
        s.setMatrix(1, e + 1, 3, Ke[e])
        s.setVector(1, e + 1, 3, O.hex8_mass_vector(dom.element_coords(e + 1), 2.0, [0, 0, -9.8]))
    _, _, val = s.getCRS()
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    ref = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=1e4, nu=0.3)
    assert np.abs(val - ref).max() <= 1e-12 * np.abs(ref).max()
    rhs_ref = O.body_force(dom.nodcoord, dom.elemnod, 2.0, [0, 0, -9.8])
    np.testing.assert_allclose(s.CRS_RHS, rhs_ref, rtol=1e-13, atol=1e-13 * np.abs(rhs_ref).max())
    # the device body-force kernel gives the same RHS
    t = solver_for(dom)
    t.assembleBodyForce(2.0, [0, 0, -9.8])
    np.testing.assert_allclose(t.CRS_RHS, rhs_ref, rtol=1e-13, atol=1e-13 * np.abs(rhs_ref).max())


def test_dirichlet_elimination_bit_exact(cuda):
    p = problems.lognormal(6, seed=11)
    dom = p["domain"]
    s = solver_for(dom)
    s.assembleStiffness(p["E"], p["nu"])
    rp, ci, val_gpu = s.getCRS()
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    s.itrmax = 1  # only the elimination matters here
    s.solve()
    rp2, ci2, val_after = s.getCRS()
    val, b = val_gpu.copy(), p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    np.testing.assert_array_equal(val_after, val)
    np.testing.assert_array_equal(s.CRS_RHS, b)


def test_crs_spmv_reference_signature(cuda):
    import scipy.sparse as sp
    rng = np.random.default_rng(0)
    for n, dens in ((1, 1.0), (50, 0.1), (3000, 0.01)):
        A = (sp.random(n, n, density=dens, random_state=n, format="csr") + sp.eye(n, format="csr")).tocsr()
        rp, ci = (A.indptr + 1).astype(np.int64), (A.indices + 1).astype(np.int32)
        x = rng.standard_normal(n)
        y0 = rng.standard_normal(n)
        y = crs_spmv_real64(A.data, rp, ci, x, y0.copy())
        yr = y0.copy()
        O.crs_spmv_real64(A.data.copy(), rp, ci, x, yr)
        assert np.abs(y - yr).max() <= 1e-13 * (np.abs(A) @ np.abs(x) + np.abs(y0)).max()
        y32 = crs_spmv_real32(A.data.astype(np.float32), rp, ci, x.astype(np.float32), np.zeros(n, np.float32))
        ref32 = A.astype(np.float32).astype(np.float64) @ x.astype(np.float32).astype(np.float64)
        assert np.abs(y32 - ref32).max() <= 1e-5 * (np.abs(A) @ np.abs(x)).max()
    # rows without entries and an empty matrix row at the end
    rp = np.array([1, 1, 3, 3], np.int64)
    ci = np.array([1, 3], np.int32)
    y = crs_spmv_real64(np.array([2.0, 3.0]), rp, ci, np.array([1.0, 5.0, 7.0]), np.ones(3))
    np.testing.assert_array_equal(y, [1.0, 24.0, 1.0])


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("algorithm,precision,pc", [("CG", "fp64", "BlockJacobi"), ("CG", "fp64", None),
                                                    ("CG", "mixed", "BlockJacobi"), ("CG", "mixed", "Jacobi"),
                                                    ("BiCGSTAB", "fp64", None), ("BiCGSTAB", "mixed", None)])
def test_solve_golden_cube4(cuda, algorithm, precision, pc):
    g = np.load(os.path.join(GOLD, "cube4_lognormal.npz"))
    dom = FEMDomain().create("Cube3D", 4, 4, 4)
    s = solver_for(dom)
    s.assembleStiffness(g["E"], 0.3)
    s.setRHS(g["rhs_in"])
    s.fix(1, np.nonzero(g["fixed"])[0] + 1, FixValue=0.0)
    s.relative_er = 1e-12
    x = s.solve(algorithm=algorithm, preconditioning=pc, precision=precision, stop_rule="true_relative")
    assert s.last_info["status"] == 0
    assert s.last_info["rel_residual"] <= 1e-12
    assert _rel(x, g["x"]) <= 1e-8


@pytest.mark.parametrize("update_mode", [1, 2])
@pytest.mark.parametrize("algorithm,precision,pc", [("CG", "fp64", "BlockJacobi"), ("CG", "mixed", "BlockJacobi"),
                                                    ("BiCGSTAB", "mixed", None), ("BiCGSTAB", "fp64", None),
                                                    ("BiCGSTAB", "mixed", "BlockJacobi"),
                                                    ("BiCGSTAB", "fp64", "Jacobi")])
def test_solve_vs_fp64_oracle(cuda, algorithm, precision, pc, update_mode):
    """Displacement within 1e-8 of the FP64 oracle solved to 1e-12."""
    p = problems.lognormal(12)
    dom = p["domain"]
    rp, ci, val, b = oracle_system(dom, p["E"], p["nu"], p["rhs"], p["fix_ids"])
    xo, rc, it, rr = O.pcg(rp, ci, val, b, tol=1e-12)
    assert rc == 0
    s = solver_for(dom)
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    s.relative_er = 1e-12
    x = s.solve(algorithm=algorithm, preconditioning=pc, precision=precision, stop_rule="true_relative",
                update_mode=update_mode)
    assert s.last_info["status"] == 0, s.last_info
    assert _rel(x, xo) <= 1e-8, (_rel(x, xo), s.last_info)


@pytest.mark.parametrize("algorithm,pc", [("BiCGSTAB", None), ("CG", "BlockJacobi")])
def test_mixed_reaches_1e10_on_larger_mesh(cuda, algorithm, pc):
    """Size-independent check at 30^3 (89k DOF): the mixed solve reaches a
    1e-10 FP64 residual and agrees with the FP64 GPU solve to 1e-8."""
    p = problems.lognormal(30)
    s = solver_for(p["domain"])
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    s.relative_er = 1e-12
    x64 = s.solve(algorithm="CG", preconditioning="BlockJacobi", precision="fp64", stop_rule="true_relative")
    assert s.last_info["status"] == 0
    s.relative_er = 1e-10
    xm = s.solve(algorithm=algorithm, preconditioning=pc, precision="mixed", stop_rule="true_relative")
    assert s.last_info["status"] == 0 and s.last_info["rel_residual"] <= 1e-10, s.last_info
    assert _rel(xm, x64) <= 1e-7, (_rel(xm, x64), s.last_info)


def test_reference_bicgstab_matches_oracle(cuda):
    """Default solve() = bicgstab_CRS_2 with the reference stop rule."""
    p = problems.cube(6)
    dom = p["domain"]
    rp, ci, val, b = oracle_system(dom, p["E"], p["nu"], p["rhs"], p["fix_ids"])
    xo, rc, ito = O.bicgstab_crs2(rp, ci, val, b)
    assert rc == 0
    s = solver_for(dom)
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    x = s.solve()
    assert s.last_info["status"] == 0
    # same algorithm and stop rule; rounding differs (parallel dot products),
    # so the iteration counts agree only to a few iterations
    assert abs(s.last_info["iterations"] - ito) <= max(5, 0.15 * ito)
    assert _rel(x, xo) <= 1e-8


def test_gravity_bar_kat_gpu(cuda):
    """benchmark_bar_in_gravity_field.f90 through the GPU path: I1 of the
    bottom element -234.026 on the deformed mesh (theory -234.024)."""
    dom = FEMDomain().create("Cube3D", 10, 10, 100)
    dom.resize(z=10.0)
    s = solver_for(dom)
    s.assembleStiffness(2.17e7, 0.0)
    s.assembleBodyForce(2.4, [0.0, 0.0, -9.8])
    for d in (2, 1, 0):
        s.fix(1, dom.select(z_max=dom.z_min()) * 3 - d, FixValue=0.0)
    x = s.solve()
    assert s.last_info["status"] == 0
    S = O.element_stress(dom.nodcoord + x.reshape(-1, 3), dom.elemnod, x, 2.17e7, 0.0)
    assert abs(np.trace(S[0]) - (-234.026)) < 1e-3


def test_poisson_scalar_crs_path(cuda):
    """FEMSolver_PoissonMatrix.f90: setCRS(CRS) with a scalar (1x1-block) matrix."""
    import scipy.sparse as sp
    n = 100
    A = sp.diags([np.full(n - 1, -1.0), np.full(n, 2.0), np.full(n - 1, -1.0)], [-1, 0, 1]).tolil()
    A[0, :] = 0.0
    A[:, 0] = 0.0
    A[0, 0] = 1.0
    A = A.tocsr()
    A.eliminate_zeros()
    rhs = np.zeros(n)
    rhs[0] = rhs[1] = 10.0
    s = FEMSolver()
    s.setCRS(CRS=((A.indptr + 1).astype(np.int64), (A.indices + 1).astype(np.int32), A.data))
    s.setRHS(rhs)
    s.relative_er = 1e-12
    x = s.solve(algorithm="CG", stop_rule="true_relative")
    exact = np.linalg.solve(A.toarray(), rhs)
    assert _rel(x, exact) < 1e-9


def test_linear_solver_plugin(cuda):
    p = problems.lognormal(8, seed=5)
    dom = p["domain"]
    rp, ci, val, b = oracle_system(dom, p["E"], p["nu"], p["rhs"], p["fix_ids"])
    xo, rc, it, rr = O.pcg(rp, ci, val, b, tol=1e-12)
    # repeated calls reuse the cached context and its captured graphs; a
    # system of another size in between must not leave stale pointers behind
    q = problems.cube(5)
    rq, cq, vq, bq = oracle_system(q["domain"], q["E"], q["nu"], q["rhs"], q["fix_ids"])
    for prec in ("fp64", "mixed", "mixed", "fp64"):
        x = np.zeros(b.shape[0])
        info = linear_solver_crs(rp, ci, val, b, x, algorithm="CG", precision=prec, relative_er=1e-12)
        assert info["status"] == 0 and _rel(x, xo) <= 1e-8
        xq = np.zeros(bq.shape[0])
        assert linear_solver_crs(rq, cq, vq, bq, xq, algorithm="CG", precision=prec, relative_er=1e-10)["status"] == 0


def test_solve_is_deterministic(cuda):
    p = problems.lognormal(10, seed=8)
    xs = []
    for _ in range(2):
        s = solver_for(p["domain"])
        s.assembleStiffness(p["E"], p["nu"])
        s.setRHS(p["rhs"])
        s.fix(1, p["fix_ids"], FixValue=0.0)
        xs.append(s.solve(algorithm="CG", preconditioning="BlockJacobi", precision="mixed",
                          stop_rule="true_relative"))
    np.testing.assert_array_equal(xs[0], xs[1])


def test_error_codes(cuda):
    dom = FEMDomain().create("Cube3D", 2, 2, 2)
    s = FEMSolver()
    with pytest.raises(_native.NativeError) as e:
        s.solve()
    assert e.value.code == -2  # PFG_E_STATE: solve before setCRS
    s.setDomain(dom)
    s.setCRS(3)
    with pytest.raises(_native.NativeError) as e:
        s.setMatrix(1, dom.ne() + 1, 3, np.zeros((24, 24)))
    assert e.value.code == -1
    with pytest.raises(_native.NativeError) as e:
        s.assembleStiffness(np.full(dom.ne(), np.nan), 0.3)
    assert e.value.code == -10
    flat = FEMDomain().create("Cube3D", 2, 2, 2)
    flat.nodcoord[:, 2] = 0.0  # zero-volume elements
    t = solver_for(flat)
    with pytest.raises(_native.NativeError) as e:
        t.assembleStiffness(1e4, 0.3)
    assert e.value.code == -7  # PFG_E_DETJ
    # out-of-range fix ids are skipped like the reference's first fix call
    s.assembleStiffness(1e4, 0.3)
    s.fix(1, np.array([0, -3, 10 ** 6, 1], np.int32), FixValue=0.0)

"""Symmetric (upper-half) FP32 storage of the mixed solves.

The mixed inner iterations may read only the upper 3x3 blocks of a symmetric
matrix, applying each strictly-upper block also transposed.  Checked here:
the solves agree with the FP64 oracle (CPU Jacobi-CG to 1e-13) to 1e-8 and
with the full-storage mixed solve; the product itself equals the full FP32
product to FP32 rounding; the mixed BiCGSTAB from the upper half (fixed-point
transposes) is bitwise reproducible; an unsymmetric matrix is refused with
PFG_E_ARG.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from plantfem_gb300 import FEMDomain, FEMSolver, problems
from plantfem_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _system(n=10, seed=20261203):
    p = problems.lognormal(n, seed=seed)
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=p["E"], nu=p["nu"])
    b = p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    xo, rc, _, _ = O.pcg(rp, ci, val, b, tol=1e-13)
    assert rc == 0
    return p, xo


def _solver(p):
    s = FEMSolver()
    s.setDomain(p["domain"])
    s.setCRS(3)
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    return s


@pytest.mark.parametrize("algorithm,pc", [("CG", "BlockJacobi"), ("CG", "Jacobi"), ("CG", None),
                                          ("BiCGSTAB", "BlockJacobi"), ("BiCGSTAB", None)])
def test_symmetric_storage_matches_oracle(cuda, algorithm, pc):
    p, xo = _system()
    s = _solver(p)
    s.relative_er = 1e-12
    x = s.solve(algorithm=algorithm, preconditioning=pc, precision="mixed", stop_rule="true_relative",
                storage="symmetric")
    assert s.last_info["status"] == 0, s.last_info
    assert s.last_info["rel_residual"] <= 1e-12
    assert _rel(x, xo) <= 1e-8, _rel(x, xo)
    xf = s.solve(algorithm=algorithm, preconditioning=pc, precision="mixed", stop_rule="true_relative")
    assert _rel(x, xf) <= 1e-9


@pytest.mark.parametrize("pc", ["BlockJacobi", None])
def test_symmetric_cg_fused_direction_matches_oracle(cuda, pc):
    """update_mode "fused": the direction update p = z + beta p rides in the
    symmetric product (ping-pong p buffers); same bar as the separate form."""
    p, xo = _system(12, seed=9)
    s = _solver(p)
    s.relative_er = 1e-12
    x = s.solve(algorithm="CG", preconditioning=pc, precision="mixed", stop_rule="true_relative",
                storage="symmetric", update_mode="fused")
    assert s.last_info["status"] == 0 and s.last_info["fallback"] == 0, s.last_info
    assert _rel(x, xo) <= 1e-8, _rel(x, xo)


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("algorithm", ["CG", "BiCGSTAB"])
def test_symmetric_storage_tiny_meshes(cuda, n, algorithm):
    """One partial slice (8, 27 or 64 nodes: fewer block rows than the 32 of a
    slice, most warps of the staged products without a slice): the
    shared-memory staging still matches the oracle."""
    p, xo = _system(n, seed=100 + n)
    s = _solver(p)
    s.relative_er = 1e-12
    x = s.solve(algorithm=algorithm, preconditioning="BlockJacobi", precision="mixed", stop_rule="true_relative",
                storage="symmetric")
    assert s.last_info["status"] == 0, s.last_info
    assert _rel(x, xo) <= 1e-8, _rel(x, xo)


def test_symmetric_storage_larger_mesh_twice(cuda):
    """30^3: two symmetric-storage mixed CG solves in a row reach 1e-10 and
    agree with the FP64 GPU solve to 1e-8 (the second reuses the upper copy)."""
    p = problems.lognormal(30)
    s = _solver(p)
    s.relative_er = 1e-10
    x64 = s.solve(algorithm="CG", preconditioning="BlockJacobi", precision="fp64", stop_rule="true_relative")
    for _ in range(2):
        xm = s.solve(algorithm="CG", preconditioning="BlockJacobi", precision="mixed", stop_rule="true_relative",
                     storage="symmetric")
        assert s.last_info["status"] == 0 and s.last_info["rel_residual"] <= 1e-10, s.last_info
        assert _rel(xm, x64) <= 1e-8


def test_symmetric_product_profiles(cuda):
    """The profiled symmetric product runs and reports half the matrix bytes
    of the full product (kernels 7, 8 of pfg_profile_kernel; 11 is 8 without
    the shared-memory staging)."""
    p, _ = _system(8)
    s = _solver(p)
    s.eliminate()
    lib = N.load()
    got = {}
    for kid in (1, 7, 8, 11):
        ms, by = C.c_double(), C.c_double()
        N.check(lib.pfg_profile_kernel(s.handle, kid, 3, C.byref(ms), C.byref(by)))
        got[kid] = by.value
        assert ms.value > 0.0
    assert got[7] == got[8] == got[11] and 0.45 * got[1] < got[7] < 0.65 * got[1]


@pytest.mark.parametrize("pc", ["BlockJacobi", None])
def test_symmetric_bicgstab_is_bitwise_reproducible(cuda, pc):
    """Mixed BiCGSTAB from the upper half: the transposes are summed in 64-bit
    fixed point, so repeated solves (same solver, then a fresh one) give the
    same iterations and the same bits, and agree with the oracle to 1e-8."""
    p, xo = _system(12, seed=5)
    runs = []
    s = None
    for fresh in (True, False, True):
        s = _solver(p) if fresh else s
        s.relative_er = 1e-12
        x = s.solve(algorithm="BiCGSTAB", preconditioning=pc, precision="mixed", stop_rule="true_relative",
                    storage="symmetric")
        assert s.last_info["status"] == 0 and s.last_info["fallback"] == 0, s.last_info
        assert _rel(x, xo) <= 1e-8
        runs.append((x, s.last_info["iterations"], s.last_info["replacements"]))
    for x, it, rep in runs[1:]:
        assert (it, rep) == runs[0][1:]
        np.testing.assert_array_equal(x, runs[0][0])


def test_fixed_point_product_profiles(cuda):
    """Kernel 10 (the BiCGSTAB product from the upper half) runs and reports the
    upper half's bytes, like kernel 7."""
    p, _ = _system(8)
    s = _solver(p)
    s.eliminate()
    lib = N.load()
    got = {}
    for kid in (7, 10):
        ms, by = C.c_double(), C.c_double()
        N.check(lib.pfg_profile_kernel(s.handle, kid, 3, C.byref(ms), C.byref(by)))
        got[kid] = by.value
        assert ms.value > 0.0
    assert got[7] == got[10]


def test_unsymmetric_matrix_is_refused(cuda):
    """A 3x3-block matrix whose (0,1) block differs from the transpose of its
    (1,0) block: symmetric storage answers PFG_E_ARG, full storage solves."""
    dom = FEMDomain().create("Cube3D", 3, 3, 3)
    p = {"domain": dom, "E": np.full(dom.ne(), 1e4), "nu": np.full(dom.ne(), 0.3)}
    s = FEMSolver()
    s.setDomain(dom)
    s.setCRS(3)
    s.assembleStiffness(p["E"], p["nu"])
    rp, ci, val = s.getCRS()
    val = val.copy()
    # scalar row 1 (node 1, x), column 4 (node 2, x): perturb one side only
    k = [q for q in range(rp[0] - 1, rp[1] - 1) if ci[q] == 4][0]
    val[k] *= 1.5
    t = FEMSolver()
    t.setCRS(CRS=(rp, ci, val))
    rhs = np.ones(rp.shape[0] - 1)
    t.setRHS(rhs)
    n = rp.shape[0] - 1
    t.fix(1, np.arange(n - 11, n + 1, dtype=np.int32), FixValue=0.0)  # far from the perturbed block
    with pytest.raises(N.NativeError) as e:
        t.solve(algorithm="BiCGSTAB", preconditioning="BlockJacobi", precision="mixed", stop_rule="true_relative",
                storage="symmetric")
    assert e.value.code == -1

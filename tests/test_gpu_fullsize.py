"""Size-independent checks on the benchmark system itself (3,090,903 DOF).

The oracle cannot solve the 100^3 lognormal cube in test time, so at full size
the solves are checked through properties that do not depend on it:
  * the true relative residual |b - K x| / |b| <= 1e-10, recomputed here with
    an independent SpMV (the sliced FP64 product, not the solver's residual);
  * the mixed-precision (symmetric FP32 copy) and FP64 solutions agree to
    1e-8 relative displacement error, the path's accuracy bar;
  * the fixed DOFs are exactly zero in every solution (elimination and restore);
  * mixed-precision BiCGSTAB (block Jacobi, symmetric FP32 copy) reaches the
    FP64 CG displacement to 1e-8.
"""
import numpy as np
import pytest
import torch

from plantfem_gb300 import FEMSolver, problems

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def system():
    p = problems.lognormal(100)
    s = FEMSolver()
    s.setDomain(p["domain"])
    s.setCRS(3)
    s.assembleStiffness(p["E"], p["nu"])
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    s.relative_er = TOL
    s.itrmax = 20000
    s.eliminate()
    b = torch.tensor(s.CRS_RHS, dtype=torch.float64, device="cuda")
    return s, p, b


def _solve(s, b, **kw):
    x = torch.zeros_like(b)
    info = s.solve_device(b, x, stop_rule="true_relative", **kw)
    assert info["status"] == 0, info
    return x, info


def _true_rel(s, b, x):
    y = torch.empty_like(b)
    s.matvec_device(x, y)
    return float(torch.linalg.norm(b - y) / torch.linalg.norm(b))


def test_fullsize_mixed_vs_fp64_cg(cuda, system):
    s, p, b = system
    assert b.shape[0] == 3 * 101 ** 3
    x64, i64 = _solve(s, b, algorithm="CG", preconditioning="BlockJacobi", precision="fp64")
    xm, im = _solve(s, b, algorithm="CG", preconditioning="BlockJacobi", precision="mixed", storage="symmetric")
    assert _true_rel(s, b, x64) <= TOL and _true_rel(s, b, xm) <= TOL
    assert float(torch.linalg.norm(xm - x64) / torch.linalg.norm(x64)) <= 1e-8
    fixed = torch.tensor(p["fix_ids"] - 1, device="cuda")
    assert torch.all(x64[fixed] == 0) and torch.all(xm[fixed] == 0)


def test_fullsize_bicgstab_matches_cg(cuda, system):
    s, p, b = system
    x64, _ = _solve(s, b, algorithm="CG", preconditioning="BlockJacobi", precision="fp64")
    xb, ib = _solve(s, b, algorithm="BiCGSTAB", preconditioning="BlockJacobi", precision="mixed",
                    storage="symmetric")
    assert _true_rel(s, b, xb) <= TOL
    assert float(torch.linalg.norm(xb - x64) / torch.linalg.norm(x64)) <= 1e-8

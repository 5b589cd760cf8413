"""saveMatrix / loadMatrix through the GPU handle (FEMSolverClass.f90:1203-1306)."""
import numpy as np
import pytest

from plantfem_gb300 import FEMSolver, problems
from plantfem_gb300.crs_io import read_crs_files

pytestmark = pytest.mark.gpu


def test_save_read_solve_and_load(cuda, tmp_path):
    p = problems.lognormal(5, seed=9)
    s = FEMSolver()
    s.setDomain(p["domain"])
    s.setCRS(3)
    s.assembleStiffness(p["E"], p["nu"])
    s.keepThisMatrixAs("A")
    name = str(tmp_path / "K")
    s.saveMatrix(name)
    rp, ci, v = s.getCRS()
    r2, c2, v2 = read_crs_files(name)
    assert np.array_equal(r2, rp) and np.array_equal(c2, ci) and np.array_equal(v2, v)
    # a plantFEM-saved matrix handed back through setCRS(CRS) solves the same system
    s.setRHS(p["rhs"])
    s.fix(1, p["fix_ids"], FixValue=0.0)
    s.relative_er = 1e-12
    x1 = s.solve(algorithm="CG", preconditioning="BlockJacobi", stop_rule="true_relative")
    t = FEMSolver()
    t.setCRS(CRS=(r2, c2, v2))
    t.setRHS(p["rhs"])
    t.fix(1, p["fix_ids"], FixValue=0.0)
    t.relative_er = 1e-12
    x2 = t.solve(algorithm="CG", preconditioning="BlockJacobi", stop_rule="true_relative")
    assert np.linalg.norm(x1 - x2) <= 1e-10 * np.linalg.norm(x1)
    # loadMatrix("A") restores the kept (uneliminated) matrix
    s.zeros()
    s.loadMatrix("A")
    r3, c3, v3 = s.getCRS()
    assert np.array_equal(r3, rp) and np.array_equal(c3, ci) and np.array_equal(v3, v)


def test_vtk_mesh_in_solves_like_the_original(cuda, tmp_path):
    """A mesh written by FEMDomain.vtk and read back by importVTKFile assembles
    and solves to the same displacement as the domain it came from."""
    from plantfem_gb300 import FEMDomain
    p = problems.lognormal(5, seed=4)
    dom = p["domain"]
    dom.vtk(str(tmp_path / "organ"))
    back = FEMDomain().importVTKFile(str(tmp_path / "organ.vtk"))
    xs = []
    for d in (dom, back):
        s = FEMSolver()
        s.setDomain(d)
        s.setCRS(3)
        s.assembleStiffness(p["E"], p["nu"])
        s.setRHS(p["rhs"])
        s.fix(1, p["fix_ids"], FixValue=0.0)
        s.relative_er = 1e-12
        xs.append(s.solve(algorithm="CG", preconditioning="BlockJacobi", stop_rule="true_relative"))
    assert np.array_equal(xs[0], xs[1])

"""plantfem_gb300 -- GB300-native (sm_103a) linear-elastic hex8 solve path of plantFEM.

The compute lives in ``libpfg.so`` (CUDA kernels + C ABI, ``include/pfg.h``);
this package is the thin Python side of that ABI:

* :class:`FEMDomain` -- structured hex8 meshes (``Cube3D``), selection;
* :class:`FEMSolver` -- plantFEM's ``FEMSolver_`` call surface;
* :class:`FEMSolverBatch` -- many FEMSolver systems in one persistent launch;
* :class:`SeismicAnalysis` -- modal analysis, linear Newmark-beta time stepping with Rayleigh damping;
* :class:`ModalAnalysis` -- plantFEM's ``ModalAnalysis_`` (eigenfrequencies and modes);
* :mod:`problems` -- the benchmark problems (meshes, loads, boundary conditions);
* :func:`build` -- compile the library in-tree.
"""
from .femdomain import FEMDomain
from .femsolver import FEMSolver, crs_spmv_real32, crs_spmv_real64, linear_solver_crs
from .batch import FEMSolverBatch
from .seismic import SeismicAnalysis
from .modal import ModalAnalysis
from . import problems


def build(verbose: bool = False) -> str:
    from .build import build as _b
    return _b(verbose=verbose)


__all__ = ["FEMDomain", "FEMSolver", "FEMSolverBatch", "SeismicAnalysis", "ModalAnalysis", "crs_spmv_real64", "crs_spmv_real32", "linear_solver_crs", "problems",
           "build"]

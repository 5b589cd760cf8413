"""FEMSolver: plantFEM's ``FEMSolver_`` call surface over the GPU library.

Every method maps to one C-ABI entry point of ``include/pfg.h`` (see there
for the reference line each replaces).  Public fields keep the reference's
names and defaults (FEMSolverClass.f90:69-76).  Ids are 1-based as in the
reference; arrays are numpy float64 / int32 / int64.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .femdomain import FEMDomain


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _torch_sync():
    import torch
    torch.cuda.current_stream().synchronize()


class FEMSolver:
    # FEMSolver_ public configuration (FEMSolverClass.f90:69-76)
    itrmax: int = 100000
    er0: float = 1.0e-10
    relative_er: float = 1.0e-10
    debug: bool = False
    use_LOBPCG: bool = False
    LOBPCG_MAX_ITR: int = 100000
    LOBPCG_TOL: float = 1.0e-6
    LOBPCG_NUM_MODE: int = 5

    def __init__(self, NumDomain: int = 1):
        self._lib = N.load()
        self._h = C.c_void_p()
        self.init(NumDomain)

    # ------------------------------------------------------------- lifecycle
    def init(self, NumDomain: int = 1):
        """FEMSolver_%init (FEMSolverClass.f90:174-327); one domain on this path."""
        if NumDomain != 1:
            raise NotImplementedError("multi-domain (overset) solves are outside this path")
        if self._h:
            self.remove()
        N.check(self._lib.pfg_create(C.byref(self._h)))
        self.domain = None
        self.last_info = None

    def remove(self):
        """FEMSolver_%remove (FEMSolverClass.f90:1827-1889)."""
        if getattr(self, "_h", None):
            self._lib.pfg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.remove()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------- problem
    def setDomain(self, FEMDomain: FEMDomain, DomainID: int = 1):
        """FEMSolver_%setDomain (FEMSolverClass.f90:329-419)."""
        if DomainID != 1:
            raise NotImplementedError("DomainID must be 1")
        dom = FEMDomain
        xyz = _f64(np.asfortranarray(dom.nodcoord).T.reshape(-1))  # NodCoord(nn,3) column-major
        en = _i32(np.asfortranarray(dom.elemnod).T.reshape(-1))    # ElemNod(ne,8) column-major
        N.check(self._lib.pfg_set_mesh(self._h, dom.nn(), N.ptr(xyz), dom.ne(), 8, N.ptr(en)))
        self.domain = dom

    def setCRS(self, DOF=3, CRS=None):
        """FEMSolver_%setCRS(DOF) (FEMSolverClass.f90:439) or setCRS(CRS_) (:421)."""
        if CRS is not None:
            row_ptr, col_idx, val = CRS
            rp, ci, v = _i64(row_ptr), _i32(col_idx), _f64(val)
            N.check(self._lib.pfg_set_crs_arrays(self._h, rp.shape[0] - 1, N.ptr(rp), N.ptr(ci), N.ptr(v)))
            return
        if not isinstance(DOF, (int, np.integer)):
            return self.setCRS(CRS=DOF)
        N.check(self._lib.pfg_set_crs(self._h, int(DOF)))

    def getCRS(self):
        """(row_ptr int64 1-based, col_idx int32 1-based, val) of the working matrix."""
        n = C.c_int64()
        nnz = C.c_int64()
        N.check(self._lib.pfg_get_crs_size(self._h, C.byref(n), C.byref(nnz)))
        rp = np.zeros(n.value + 1, dtype=np.int64)
        ci = np.zeros(nnz.value, dtype=np.int32)
        v = np.zeros(nnz.value)
        N.check(self._lib.pfg_get_crs(self._h, N.ptr(rp), N.ptr(ci), N.ptr(v)))
        return rp, ci, v

    @property
    def CRS_Index_Row(self):
        return self.getCRS()[0]

    @property
    def CRS_Index_Col(self):
        return self.getCRS()[1]

    @property
    def CRS_val(self):
        return self.getCRS()[2]

    def ndof(self) -> int:
        n = C.c_int64()
        N.check(self._lib.pfg_get_crs_size(self._h, C.byref(n), None))
        return n.value

    def _nnz(self) -> int:
        n, nnz = C.c_int64(), C.c_int64()
        N.check(self._lib.pfg_get_crs_size(self._h, C.byref(n), C.byref(nnz)))
        return nnz.value

    def setRHS(self, RHS):
        """FEMSolver_%setRHS (FEMSolverClass.f90:431-437)."""
        r = _f64(RHS)
        N.check(self._lib.pfg_set_rhs(self._h, r.shape[0], N.ptr(r)))

    @property
    def CRS_RHS(self):
        n = self.ndof()
        r = np.zeros(n)
        N.check(self._lib.pfg_get_rhs(self._h, n, N.ptr(r)))
        return r

    def setMatrix(self, DomainID: int, ElementID: int, DOF: int, Matrix):
        """FEMSolver_%setMatrix (FEMSolverClass.f90:901-911)."""
        m = _f64(np.asarray(Matrix, dtype=np.float64).T.reshape(-1))  # column-major 24x24
        N.check(self._lib.pfg_set_matrix(self._h, DomainID, ElementID, DOF, N.ptr(m)))

    def setMatrices(self, ElementIDs, Matrices):
        ids = _i32(ElementIDs)
        mats = _f64(np.asarray(Matrices, dtype=np.float64).transpose(0, 2, 1).reshape(-1))
        N.check(self._lib.pfg_set_matrices(self._h, ids.shape[0], N.ptr(ids), N.ptr(mats)))

    def setVector(self, DomainID: int, ElementID: int, DOF: int, Vector):
        """FEMSolver_%setVector (FEMSolverClass.f90:913-920)."""
        v = _f64(Vector)
        N.check(self._lib.pfg_set_vector(self._h, DomainID, ElementID, DOF, N.ptr(v)))

    def assembleStiffness(self, YoungModulus, PoissonRatio):
        """Whole-mesh StiffnessMatrix(ElementID, E, v) + setMatrix loop, on the GPU."""
        E = _f64(np.atleast_1d(YoungModulus))
        nu = _f64(np.broadcast_to(np.atleast_1d(PoissonRatio), E.shape))
        N.check(self._lib.pfg_assemble_stiffness(self._h, E.shape[0], N.ptr(E), N.ptr(nu)))

    def assembleMass(self, Density, Lumped: bool = False):
        rho = _f64(np.atleast_1d(Density))
        N.check(self._lib.pfg_assemble_mass(self._h, rho.shape[0], N.ptr(rho), int(bool(Lumped))))

    def assembleBodyForce(self, Density, Accel):
        rho = _f64(np.atleast_1d(Density))
        a = _f64(Accel)
        N.check(self._lib.pfg_assemble_body_force(self._h, rho.shape[0], N.ptr(rho), N.ptr(a)))

    def zeros(self):
        """FEMSolver_%zeros (FEMSolverClass.f90:1310-1322)."""
        N.check(self._lib.pfg_zeros(self._h))

    def fix(self, DomainID: int = 1, IDs=None, FixValue: float | None = None, FixValues=None):
        """FEMSolver_%fix (FEMSolverClass.f90:1073-1136)."""
        ids = _i32(IDs)
        vals = None if FixValues is None else _f64(FixValues)
        N.check(self._lib.pfg_fix(self._h, ids.shape[0], N.ptr(ids), N.ptr(vals),
                                  0.0 if FixValue is None else float(FixValue)))

    # ------------------------------------------------------------- solving
    def _opts(self, algorithm, precision, preconditioning, stop_rule, update_mode=0, reliable_delta=None,
              storage="full", ilu_order="stored"):
        alg = {"BiCGSTAB": N.ALG_BICGSTAB, "CG": N.ALG_CG}[algorithm or "BiCGSTAB"]
        prec = {"fp64": N.PREC_FP64, "FP64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]
        ilu = {"stored": N.PC_ILU0, "sorted": N.PC_ILU0_SORTED}[ilu_order]
        pc = {None: N.PC_NONE, "None": N.PC_NONE, "PointJacobi": N.PC_JACOBI, "Jacobi": N.PC_JACOBI,
              "BlockJacobi": N.PC_BLOCK_JACOBI, "ILU": ilu, "incompleteLU": ilu}[preconditioning]
        if pc in (N.PC_ILU0, N.PC_ILU0_SORTED):
            alg = N.ALG_BICGSTAB  # FEMSolverClass.f90:1777-1784: ILU always runs bicgstab_CRS_ILU
        if stop_rule is None:
            stop_rule = "reference" if prec == N.PREC_FP64 else "true_relative"
        sr = {"reference": N.STOP_REFERENCE, "true_relative": N.STOP_TRUE_RELATIVE}[stop_rule]
        um = {0: 0, "auto": 0, 1: 1, "fused": 1, 2: 2, "separate": 2}[update_mode]
        o = N.default_opts(algorithm=alg, precision=prec, precond=pc, stop_rule=sr, itrmax=int(self.itrmax),
                           er0=float(self.er0), relative_er=float(self.relative_er), debug=int(bool(self.debug)),
                           update_mode=um, storage={"full": N.STORAGE_FULL, "symmetric": N.STORAGE_SYMMETRIC}[storage])
        if reliable_delta is not None:
            o.reliable_delta = float(reliable_delta)
        return o

    def solve(self, algorithm: str | None = None, preconditioning: str | None = None, x0=None,
              precision: str = "fp64", stop_rule: str | None = None, update_mode=0,
              storage: str = "full", ilu_order: str = "stored") -> np.ndarray:
        """x = FEMSolver_%solve([algorithm], [preconditioning], [x0]) (FEMSolverClass.f90:1697-1825).

        Defaults reproduce the reference: unpreconditioned BiCGSTAB in FP64 with
        its stop rule.  ``algorithm="CG"``, ``preconditioning="BlockJacobi"`` and
        ``precision="mixed"`` select the GB300 forms.  ``preconditioning="ILU"``
        (or ``"incompleteLU"``) runs bicgstab_CRS_ILU: FP64 BiCGSTAB with the
        ILU(0) factor kept on the solver; ``ilu_order="sorted"`` factors with
        each row's columns in ascending order (``"stored"``: the row's own
        order, as ILUCRS).  Breakdown raises (the reference stops); itrmax is
        reported in ``last_info``.
        """
        opts = self._opts(algorithm, precision, preconditioning, stop_rule, update_mode, storage=storage,
                          ilu_order=ilu_order)
        n = self.ndof()
        x = np.zeros(n)
        xi = None if x0 is None else _f64(x0)
        info = N.Info()
        N.check(self._lib.pfg_solve(self._h, C.byref(opts), N.ptr(xi), N.ptr(x), C.byref(info)))
        self.last_info = info.as_dict()
        return x

    def ILU(self, sorted: bool = False, RHS=None) -> np.ndarray:
        """ILUCRS(0) (SparseClass.f90:1629-1792) of the stored matrix, kept on the
        solver for ILU solves -> the factor's values on getCRS()'s pattern.
        With RHS: CRS_%ILU(0, RHS) -> the solve L U x = RHS with the factor
        (:1647-1679); the stored matrix itself is not overwritten."""
        if RHS is not None:
            N.check(self._lib.pfg_ilu_factor(self._h, int(bool(sorted)), None))
            r = _f64(RHS)
            x = np.zeros_like(r)
            N.check(self._lib.pfg_ilu_solve(self._h, N.ptr(r), N.ptr(x)))
            return x
        lu = np.zeros(self._nnz())
        N.check(self._lib.pfg_ilu_factor(self._h, int(bool(sorted)), N.ptr(lu)))
        return lu

    def ILU_matvec(self, old_vector) -> np.ndarray:
        """ILU_matvecCRS (SparseClass.f90:1795-1852) with the kept factor, as it
        executes: D^-1 L^-1 old_vector."""
        v = _f64(old_vector)
        out = np.zeros_like(v)
        N.check(self._lib.pfg_ilu_apply(self._h, N.ptr(v), N.ptr(out)))
        return out

    def resetILU(self):
        """Drop the kept ILU(0) factor (the next ILU solve factors again)."""
        N.check(self._lib.pfg_ilu_reset(self._h))

    def eliminate(self):
        """Apply the Dirichlet elimination of FEMSolver_%solve (FEMSolverClass.f90:1707-1756)
        to the stored matrix and RHS now (solve() does it itself)."""
        N.check(self._lib.pfg_eliminate(self._h))

    # option strings of getElementCauchyStress (FEMDomainClass.f90:15310-15362)
    _STRESS_OPTIONS = {**{k: 2 for k in ("p", "P")},
                       **{k: 1 for k in ("I", "I1", "i1", "trace", "tr", "TRACE", "TR")},
                       **{k: 3 for k in ("II", "I2", "i2", "ii")},
                       **{k: 4 for k in ("III", "I3", "i3", "iii")},
                       **{k: 5 for k in ("J", "J1", "j1", "j")},
                       **{k: 6 for k in ("JJ", "J2", "j2", "jj")},
                       **{k: 7 for k in ("JJJ", "J3", "j3", "jjj")},
                       **{f"{a}{i},{j}{b}": 10 + 3 * (i - 1) + (j - 1)
                          for i, j in ((1, 1), (2, 2), (3, 3)) for a, b in (("", ""), ("(", ")"), ("_{", "}"))},
                       **{f"{a}{p},{q}{b}": 10 + 3 * (i - 1) + (j - 1)
                          for i, j in ((1, 2), (1, 3), (2, 3)) for p, q in ((i, j), (j, i))
                          for a, b in (("", ""), ("(", ")"), ("_{", "}"))}}

    def getElementCauchyStress(self, displacement, E, v, i: int | None = None, j: int | None = None,
                               option: str | None = None):
        """getElementCauchyStress (FEMDomainClass.f90:15249-15370): cell-averaged
        Cauchy stress per element (StressMatrix, :11912-12035).

        * ``i, j`` given (1-based): the component sigma(i, j) of every element;
        * ``option``: one invariant or component per element -- "p", "I1" (and
          "I", "trace", ...), "I2", "I3", "J1", "J2", "J3" (of the deviator, as
          the reference computes them: J2 = (tr(s)^2 - tr(s s)) / 2), or
          "1,1" ... "3,2" in any of the reference's spellings; an option the
          reference does not know gives zeros, as its ``select case`` does;
        * neither: the (ne, 3, 3) tensors.
        """
        d = _f64(displacement)
        Ev = _f64(np.atleast_1d(E))
        vv = _f64(np.broadcast_to(np.atleast_1d(v), Ev.shape))
        ne = self.domain.ne()
        if i is not None and j is not None:
            opt = 10 + 3 * (int(i) - 1) + (int(j) - 1)
        elif option is None:
            opt = 0
        else:
            opt = self._STRESS_OPTIONS.get(option)
            if opt is None:
                return np.zeros(ne)
        out = np.zeros(ne * 9 if opt == 0 else ne)
        N.check(self._lib.pfg_element_stress(self._h, N.ptr(d), Ev.shape[0], N.ptr(Ev), N.ptr(vv), opt, N.ptr(out)))
        return out.reshape(ne, 3, 3) if opt == 0 else out

    # device-array forms (PyTorch tensors)
    def assembleStiffness_device(self, E, nu):
        _torch_sync()
        N.check(self._lib.pfg_dev_assemble_stiffness(self._h, E.numel(), E.data_ptr(), nu.data_ptr(), None))

    def setRHS_device(self, rhs):
        _torch_sync()
        N.check(self._lib.pfg_dev_set_rhs(self._h, rhs.numel(), rhs.data_ptr(), None))

    def adjoint_grad_E_device(self, u, lam, nu, grad):
        _torch_sync()
        N.check(self._lib.pfg_dev_adjoint_grad_E(self._h, u.data_ptr(), lam.data_ptr(), nu.numel(), nu.data_ptr(),
                                                 grad.data_ptr(), None))
        return grad

    # ------------------------------------------------------------ eigenproblem
    def keepThisMatrixAs(self, As: str):
        """FEMSolver_%keepThisMatrixAs (FEMSolverClass.f90:1544-1604)."""
        N.check(self._lib.pfg_keep_this_matrix_as(self._h, As.encode()))

    def loadMatrix(self, from_: str):
        """FEMSolver_%loadMatrix(from) (FEMSolverClass.f90:1203-1222): the matrix
        kept as "A" or "B" becomes the working matrix."""
        N.check(self._lib.pfg_load_matrix(self._h, from_.encode()))

    def saveMatrix(self, name: str, CRS_as_dense: bool = False, zero_or_nonzero: bool = False):
        """FEMSolver_%saveMatrix (FEMSolverClass.f90:1225-1306): the working matrix
        as name_data.txt / name_indices.txt / name_indptr.txt (one entry per
        line, 1-based indices), or as name_dense.csv."""
        from .crs_io import write_crs_files, write_dense_csv
        rp, ci, v = self.getCRS()
        if CRS_as_dense:
            write_dense_csv(name + "_dense.csv", rp, ci, v, zero_or_nonzero)
        else:
            write_crs_files(name, rp, ci, v)

    def fix_eig(self, IDs):
        """FEMSolver_%fix_eig (FEMSolverClass.f90:1607-1628)."""
        ids = _i32(IDs)
        N.check(self._lib.pfg_fix_eig(self._h, ids.shape[0], N.ptr(ids)))

    def eig(self, num_eigen: int | None = None, block_size: int = 0, precision: str = "fp64",
            preconditioning: str | None = "BlockJacobi", stop_rule: str = "residual", seed: int = 1,
            eigen_vectors: bool = True, tol_fp32: float | None = None):
        """(eigen_value, eigen_vectors) = FEMSolver_%eig (FEMSolverClass.f90:1384-1541).

        As the reference, on the matrices kept as "A" and "B" with the fix_eig
        DOFs removed, and by ``use_LOBPCG``:

        * ``use_LOBPCG = False`` (the reference's default): the dense branch
          (DSPGVD, :1470-1500) -- every eigenpair (or the lowest
          ``num_eigen``), on the GPU by pfg_eig_dense, at most 4096 unknowns;
        * ``use_LOBPCG = True``: LOBPCG (LOBPCG_CRS, SparseClass.f90:2008-2239)
          for ``num_eigen`` (default LOBPCG_NUM_MODE) pairs with LOBPCG_TOL /
          LOBPCG_MAX_ITR; ``block_size``, ``precision`` ("mixed": FP32 phase
          then FP64), ``preconditioning`` and ``stop_rule`` select its form.

        eigen_vectors: ndof x count, zero at the fixed DOFs (None with
        ``eigen_vectors=False``).
        """
        if not self.use_LOBPCG:
            return self._eig_dense(num_eigen, eigen_vectors)
        nev = int(num_eigen or self.LOBPCG_NUM_MODE)
        o = N.EigOpts()
        self._lib.pfg_eig_opts_default(C.byref(o))
        o.block_size = int(block_size)
        o.max_itr = int(self.LOBPCG_MAX_ITR)
        o.tol = float(self.LOBPCG_TOL)
        o.precision = {"fp64": N.PREC_FP64, "FP64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]
        o.precond = {None: N.PC_NONE, "None": N.PC_NONE, "Jacobi": N.PC_JACOBI, "PointJacobi": N.PC_JACOBI,
                     "BlockJacobi": N.PC_BLOCK_JACOBI}[preconditioning]
        o.stop_rule = {"reference": N.EIG_STOP_REFERENCE, "residual": N.EIG_STOP_RESIDUAL}[stop_rule]
        o.seed = int(seed)
        o.debug = int(bool(self.debug))
        if tol_fp32 is not None:
            o.tol_fp32 = float(tol_fp32)  # mixed: relative residual that ends the FP32 phase
        lam = np.zeros(nev)
        n = self.ndof()
        X = np.zeros((nev, n)) if eigen_vectors else None
        info = N.Info()
        N.check(self._lib.pfg_eig(self._h, C.byref(o), nev, N.ptr(lam), None if X is None else N.ptr(X),
                                  C.byref(info)))
        self.last_info = info.as_dict()
        return lam, (None if X is None else X.T)

    def _eig_dense(self, num_eigen, eigen_vectors=True):
        nred = C.c_int64()
        N.check(self._lib.pfg_eig_reduced_size(self._h, C.byref(nred)))
        count = nred.value if not num_eigen or num_eigen <= 0 else min(int(num_eigen), nred.value)
        lam = np.zeros(count)
        n = self.ndof()
        X = np.zeros((count, n)) if eigen_vectors else None
        info = N.Info()
        N.check(self._lib.pfg_eig_dense(self._h, int(num_eigen or 0), N.ptr(lam),
                                        None if X is None else N.ptr(X), C.byref(info)))
        self.last_info = info.as_dict()
        return lam, (None if X is None else X.T)

    def solve_device(self, b, x, algorithm="CG", preconditioning="BlockJacobi", precision="mixed",
                     stop_rule=None, stream=None, update_mode=0, reliable_delta=None, storage="full",
                     ilu_order="stored"):
        """Solve with the already-eliminated matrix on device tensors b -> x
        (x holds x0).  ``b`` and ``x`` are float64 CUDA tensors."""
        opts = self._opts(algorithm, precision, preconditioning, stop_rule, update_mode, reliable_delta, storage,
                          ilu_order)
        info = N.Info()
        if stream is None:
            _torch_sync()  # the library works on its own stream: order after the caller's writes
        N.check(self._lib.pfg_dev_solve(self._h, C.byref(opts), b.data_ptr(), x.data_ptr(), C.byref(info),
                                        None if stream is None else C.c_void_p(stream)))
        self.last_info = info.as_dict()
        return info.as_dict()

    def matvec_device(self, x, y, stream=None):
        """y = K x on device float64 tensors."""
        if stream is None:
            _torch_sync()
        N.check(self._lib.pfg_dev_spmv(self._h, x.data_ptr(), y.data_ptr(),
                                       None if stream is None else C.c_void_p(stream)))
        return y


def crs_spmv_real64(val, row_ptr, col_idx, old_vector, new_vector):
    """GPU crs_spmv_real64 with the reference signature (SparseClass-c.c:53-65):
    new_vector += A old_vector, 1-based CRS."""
    lib = N.load()
    v, rp, ci, x = _f64(val), _i64(row_ptr), _i32(col_idx), _f64(old_vector)
    assert new_vector.dtype == np.float64 and new_vector.flags["C_CONTIGUOUS"]
    N.check(lib.pfg_crs_spmv_real64(N.ptr(v), N.ptr(rp), N.ptr(ci), N.ptr(x), N.ptr(new_vector),
                                    new_vector.shape[0], ci.shape[0]))
    return new_vector


def crs_spmv_real32(val, row_ptr, col_idx, old_vector, new_vector):
    lib = N.load()
    v = np.ascontiguousarray(val, dtype=np.float32)
    rp, ci = _i64(row_ptr), _i32(col_idx)
    x = np.ascontiguousarray(old_vector, dtype=np.float32)
    assert new_vector.dtype == np.float32 and new_vector.flags["C_CONTIGUOUS"]
    N.check(lib.pfg_crs_spmv_real32(N.ptr(v), N.ptr(rp), N.ptr(ci), N.ptr(x), N.ptr(new_vector),
                                    new_vector.shape[0], ci.shape[0]))
    return new_vector


def linear_solver_crs(row_ptr, col_idx, val, rhs, x, algorithm="CG", precision="mixed",
                      preconditioning="BlockJacobi", relative_er=1e-10, itrmax=100000, stop_rule=None,
                      storage="full"):
    """The LinearSolver(row_ptr, col_idx, val, rhs, x) plug-in of FEMSolver_%solve
    (FEMSolverClass.f90:1632-1662) on the GPU; x is updated in place."""
    lib = N.load()
    s = FEMSolver.__new__(FEMSolver)
    s.itrmax, s.er0, s.relative_er, s.debug = itrmax, 1e-10, relative_er, False
    opts = FEMSolver._opts(s, algorithm, precision, preconditioning, stop_rule, storage=storage)
    rp, ci, v, b = _i64(row_ptr), _i32(col_idx), _f64(val), _f64(rhs)
    assert x.dtype == np.float64 and x.flags["C_CONTIGUOUS"]
    info = N.Info()
    N.check(lib.pfg_linear_solver_crs(N.ptr(rp), N.ptr(ci), N.ptr(v), N.ptr(b), N.ptr(x), b.shape[0], v.shape[0],
                                      C.byref(opts), C.byref(info)))
    return info.as_dict()

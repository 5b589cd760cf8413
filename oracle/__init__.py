"""CPU oracle for plantFEM's linear-elastic hex8 solve path.

TEST INFRASTRUCTURE ONLY: the checker the GPU library is compared against.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline
import this package; the product package ``plantfem_gb300`` never does.

The arithmetic lives in ``oracle.c`` (plain C, one routine per reference
routine, each citing plantFEM file:line); this module only marshals numpy
arrays through ctypes.  ``lobpcg.py`` restates ``LOBPCG_CRS`` in numpy.

Array conventions are the reference's: ``nodcoord`` is (nn, 3) and ``elemnod``
(ne, 8) in Fortran order with 1-based node ids; CRS arrays are 1-based
``row_ptr`` (int64) and ``col_idx`` (int32) in first-appearance column order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def build(with_ref: bool | None = None) -> None:
    """Compile liboracle.so, and oracle/_ref from the plantFEM checkout.

    The checkout's location comes from the ``PLANTFEM_SRC`` environment
    variable (default in ``oracle/Makefile``).  ``with_ref=None`` builds
    ``_ref`` only where that checkout exists (the make target fails quietly
    otherwise); ``True`` requires it; ``False`` skips it.
    """
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    if with_ref is False:
        return
    r = subprocess.run(["make", "-s", "-C", _HERE, "ref"], stdout=subprocess.DEVNULL,
                       stderr=None if with_ref else subprocess.DEVNULL)
    if with_ref and r.returncode != 0:
        raise RuntimeError("oracle/_ref: the plantFEM checkout named by PLANTFEM_SRC is missing")


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(_HERE, "liboracle.so")
    if not os.path.exists(path):
        build(with_ref=False)
    L = C.CDLL(path)
    L.orc_cube3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _d, _i32]
    L.orc_hex8_stiffness.argtypes = [_d, C.c_double, C.c_double, _d]
    L.orc_hex8_mass.argtypes = [_d, C.c_double, C.c_int, _d]
    L.orc_hex8_mass_vector.argtypes = [_d, C.c_double, _d, _d]
    L.orc_hex8_stress.argtypes = [_d, _d, C.c_double, C.c_double, _d]
    L.orc_element_stiffness_all.argtypes = [C.c_int64, C.c_int64, _d, _i32, _d, _d, _d]
    L.orc_element_stress_all.argtypes = [C.c_int64, C.c_int64, _d, _i32, _d, _d, _d, _d]
    for name in ("orc_zero_matrix", "orc_zero_matrix_legacy"):
        f = getattr(L, name)
        f.argtypes = [C.c_int64, C.c_int64, C.c_int, _i32, C.c_int, C.c_void_p, C.c_void_p]
        f.restype = C.c_int64
    L.orc_assemble.argtypes = [C.c_int64, C.c_int64, _d, _i32, C.c_int, _d, C.c_void_p, _i64, _i32, _d]
    L.orc_assemble_body_force.argtypes = [C.c_int64, C.c_int64, _d, _i32, _d, _d, _d]
    L.orc_set_matrix.argtypes = [_i64, _i32, _d, C.c_int64, _i32, C.c_int64, C.c_int, _d]
    L.orc_apply_fix.argtypes = [C.c_int64, _i64, _i32, _d, _d, _u8, _d]
    L.orc_crs_spmv_real64.argtypes = [_d, _i64, _i32, _d, _d, C.c_size_t, C.c_size_t]
    L.orc_sub_crs_matvec.argtypes = [C.c_int64, _i64, _i32, _d, _d, _d, C.c_int]
    L.orc_bicgstab_crs2.argtypes = [C.c_int64, _i64, _i32, _d, _d, _d, C.c_int, C.c_double,
                                    C.c_double, C.c_int, C.POINTER(C.c_int)]
    L.orc_pcg.argtypes = [C.c_int64, _i64, _i32, _d, _d, _d, C.c_int, C.c_double,
                          C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.orc_reduce_crs.argtypes = [C.c_int64, _i64, _i32, _d, C.c_int64, _i32, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
    L.orc_reduce_crs.restype = C.c_int64
    L.orc_ilu0.argtypes = [C.c_int64, _i64, _i32, _d, C.c_int]
    L.orc_ilu_apply.argtypes = [C.c_int64, _i64, _i32, _d, _d, _d]
    L.orc_ilu_solve.argtypes = [C.c_int64, _i64, _i32, _d, _d]
    L.orc_bicgstab_ilu.argtypes = [C.c_int64, _i64, _i32, _d, _d, _d, _d, C.c_int, C.c_double, C.c_double,
                                   C.POINTER(C.c_int)]
    L.orc_num_threads.restype = C.c_int
    L.orc_crs_spmm.argtypes = [C.c_int64, _i64, _i32, _d, C.c_int64, _d, _d]
    L.orc_gram_schmidt.argtypes = [C.c_int64, C.c_int64, C.c_void_p]
    L.orc_gram_schmidt_rm.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]
    _LIB = L
    return L


def ref_lib():
    """The reference's own SparseClass-c.c compiled into oracle/_ref (or None)."""
    global _REF
    if _REF is not None:
        return _REF
    path = os.path.join(_HERE, "_ref", "libsparseclass_c.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    L.crs_spmv_real64.argtypes = [_d, _i64, _i32, _d, _d, C.c_size_t, C.c_size_t]
    L.crs_spmv_real64.restype = None
    L.crs_spmv_real32.argtypes = [np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS"), _i64,
                                  _i32, np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS"),
                                  np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS"),
                                  C.c_size_t, C.c_size_t]
    L.crs_spmv_real32.restype = None
    _REF = L
    return L


def num_threads() -> int:
    return int(lib().orc_num_threads())


# --------------------------------------------------------------------------- mesh
def cube3d(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0):
    """Mesh_%create("Cube3D") (MeshClass.f90:6348-6361)."""
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    ne = nx * ny * nz
    xyz = np.zeros(nn * 3)
    en = np.zeros(ne * 8, dtype=np.int32)
    lib().orc_cube3d(nx, ny, nz, lx, ly, lz, xyz, en)
    return xyz.reshape(3, nn).T, en.reshape(8, ne).T


def _fortran_flat(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).T).reshape(-1)


# ------------------------------------------------------------------------ element
def hex8_stiffness(xe, E, nu):
    """StiffnessMatrixFEMDomain for one element; xe (8,3) -> Ke (24,24)."""
    Ke = np.zeros(576)
    if lib().orc_hex8_stiffness(np.ascontiguousarray(xe, dtype=np.float64).reshape(-1), E, nu, Ke):
        raise ValueError("detJ == 0")
    return Ke.reshape(24, 24).T.copy()


def hex8_mass(xe, rho, lumped=False):
    Me = np.zeros(576)
    if lib().orc_hex8_mass(np.ascontiguousarray(xe, dtype=np.float64).reshape(-1), rho, int(lumped), Me):
        raise ValueError("detJ == 0")
    return Me.reshape(24, 24).T.copy()


def hex8_mass_vector(xe, rho, accel):
    Fe = np.zeros(24)
    lib().orc_hex8_mass_vector(np.ascontiguousarray(xe, dtype=np.float64).reshape(-1), rho,
                               np.asarray(accel, dtype=np.float64), Fe)
    return Fe


def element_stiffness_all(nodcoord, elemnod, E, nu):
    nn, ne = nodcoord.shape[0], elemnod.shape[0]
    out = np.zeros(ne * 576)
    rc = lib().orc_element_stiffness_all(nn, ne, _fortran_flat(nodcoord, np.float64),
                                         _fortran_flat(elemnod, np.int32),
                                         np.ascontiguousarray(np.broadcast_to(E, (ne,)), dtype=np.float64),
                                         np.ascontiguousarray(np.broadcast_to(nu, (ne,)), dtype=np.float64),
                                         out)
    if rc:
        raise ValueError("detJ == 0")
    return out.reshape(ne, 24, 24).transpose(0, 2, 1).copy()


def element_stress(nodcoord, elemnod, disp, E, nu):
    """Cell-averaged Cauchy stress per element (ne, 3, 3)."""
    nn, ne = nodcoord.shape[0], elemnod.shape[0]
    out = np.zeros(ne * 9)
    rc = lib().orc_element_stress_all(nn, ne, _fortran_flat(nodcoord, np.float64),
                                      _fortran_flat(elemnod, np.int32),
                                      np.ascontiguousarray(disp, dtype=np.float64),
                                      np.ascontiguousarray(np.broadcast_to(E, (ne,)), dtype=np.float64),
                                      np.ascontiguousarray(np.broadcast_to(nu, (ne,)), dtype=np.float64), out)
    if rc:
        raise ValueError("detJ == 0")
    return out.reshape(ne, 3, 3)


# ------------------------------------------------------------------------ pattern
def zero_matrix(nn, elemnod, dof=3, legacy=False):
    """ZeroMatrix_as_CRS (FEMDomainClass.f90:10581-10840) -> (row_ptr, col_idx)."""
    f = lib().orc_zero_matrix_legacy if legacy else lib().orc_zero_matrix
    ne = elemnod.shape[0]
    en = _fortran_flat(elemnod, np.int32)
    nnz = f(nn, ne, 8, en, dof, None, None)
    row_ptr = np.zeros(nn * dof + 1, dtype=np.int64)
    col_idx = np.zeros(nnz, dtype=np.int32)
    f(nn, ne, 8, en, dof, row_ptr.ctypes.data, col_idx.ctypes.data)
    return row_ptr, col_idx


def assemble(nodcoord, elemnod, row_ptr, col_idx, kind="stiffness", E=None, nu=None, rho=None):
    """Serial element loop + setValue scatter (FEMSolverClass.f90:1020-1057)."""
    nn, ne = nodcoord.shape[0], elemnod.shape[0]
    val = np.zeros(col_idx.shape[0])
    if kind == "stiffness":
        p0 = np.ascontiguousarray(np.broadcast_to(E, (ne,)), dtype=np.float64)
        p1 = np.ascontiguousarray(np.broadcast_to(nu, (ne,)), dtype=np.float64)
        rc = lib().orc_assemble(nn, ne, _fortran_flat(nodcoord, np.float64), _fortran_flat(elemnod, np.int32),
                                0, p0, p1.ctypes.data, row_ptr, col_idx, val)
    else:
        p0 = np.ascontiguousarray(np.broadcast_to(rho, (ne,)), dtype=np.float64)
        rc = lib().orc_assemble(nn, ne, _fortran_flat(nodcoord, np.float64), _fortran_flat(elemnod, np.int32),
                                1, p0, None, row_ptr, col_idx, val)
    if rc:
        raise ValueError(f"assembly failed ({rc})")
    return val


def body_force(nodcoord, elemnod, rho, accel):
    nn, ne = nodcoord.shape[0], elemnod.shape[0]
    rhs = np.zeros(nn * 3)
    lib().orc_assemble_body_force(nn, ne, _fortran_flat(nodcoord, np.float64), _fortran_flat(elemnod, np.int32),
                                  np.ascontiguousarray(np.broadcast_to(rho, (ne,)), dtype=np.float64),
                                  np.asarray(accel, dtype=np.float64), rhs)
    return rhs


# ----------------------------------------------------------------------- solving
def apply_fix(row_ptr, col_idx, val, rhs, fixed_mask, fix_values):
    """BC elimination of FEMSolver_%solve (FEMSolverClass.f90:1707-1756); in place."""
    lib().orc_apply_fix(rhs.shape[0], row_ptr, col_idx, val, rhs,
                        np.ascontiguousarray(fixed_mask, dtype=np.uint8),
                        np.ascontiguousarray(fix_values, dtype=np.float64))


def spmv(row_ptr, col_idx, val, x, atomic=False):
    n = row_ptr.shape[0] - 1
    y = np.zeros(n)
    lib().orc_sub_crs_matvec(n, row_ptr, col_idx, val, np.ascontiguousarray(x, dtype=np.float64), y,
                             int(atomic))
    return y


def crs_spmv_real64(val, row_ptr, col_idx, old_vector, new_vector):
    """Restated SparseClass-c.c:53-65 (accumulates into new_vector)."""
    lib().orc_crs_spmv_real64(val, row_ptr, col_idx, old_vector, new_vector, new_vector.shape[0],
                              col_idx.shape[0])


def bicgstab_crs2(row_ptr, col_idx, val, b, x0=None, itrmax=100000, er0=1e-10, relative_er=1e-10,
                  atomic=False):
    """bicgstab_CRS_2 (FEMSolverClass.f90:2199-2298) -> (x, rc, iterations)."""
    n = b.shape[0]
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(0)
    rc = lib().orc_bicgstab_crs2(n, row_ptr, col_idx, val, x, np.ascontiguousarray(b, dtype=np.float64),
                                 itrmax, er0, relative_er, int(atomic), C.byref(it))
    return x, rc, it.value


def ilu0(row_ptr, col_idx, val, sorted=False):
    """ILUCRS(0) (SparseClass.f90:1629-1792) of a 1-based CRS -> factor values
    on the same pattern (unit lower L strictly below, U on and above the
    diagonal).  sorted=False visits each row's k in stored column order, as
    the reference does; sorted=True in ascending column order."""
    lu = np.array(val, dtype=np.float64)
    lib().orc_ilu0(row_ptr.shape[0] - 1, row_ptr, col_idx, lu, int(bool(sorted)))
    return lu


def ilu_apply(row_ptr, col_idx, lu, v):
    """ILU_matvecCRS (SparseClass.f90:1795-1852) as executed: D^-1 L^-1 v."""
    out = np.zeros(row_ptr.shape[0] - 1)
    lib().orc_ilu_apply(out.shape[0], row_ptr, col_idx, lu, np.ascontiguousarray(v, dtype=np.float64), out)
    return out


def ilu_solve(row_ptr, col_idx, lu, rhs):
    """ILUCRS(0, RHS) (SparseClass.f90:1647-1679) with the factor lu -> the solution."""
    x = np.array(rhs, dtype=np.float64)
    lib().orc_ilu_solve(x.shape[0], row_ptr, col_idx, lu, x)
    return x


def bicgstab_ilu(row_ptr, col_idx, val, b, lu=None, sorted=False, x0=None, itrmax=100000, er0=1e-10,
                 relative_er=1e-10):
    """bicgstab_CRS_ILU (LinearSolverClass.f90:4104-4230) -> (x, rc, iterations)."""
    n = b.shape[0]
    if lu is None:
        lu = ilu0(row_ptr, col_idx, val, sorted)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(0)
    rc = lib().orc_bicgstab_ilu(n, row_ptr, col_idx, val, lu, x, np.ascontiguousarray(b, dtype=np.float64),
                                itrmax, er0, relative_er, C.byref(it))
    return x, rc, it.value


def spmm(row_ptr, col_idx, val, X):
    """Y = A X for a block of vectors X (n x m), the oracle's CRS_%matmul per column."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = row_ptr.shape[0] - 1
    Y = np.empty((n, X.shape[1]))
    lib().orc_crs_spmm(n, row_ptr, col_idx, val, X.shape[1], X.reshape(-1), Y.reshape(-1))
    return Y


class CrsOperator:
    """A 1-based CRS matrix usable as ``A @ X`` in ``oracle.lobpcg`` (OpenMP products)."""

    def __init__(self, row_ptr, col_idx, val):
        self.row_ptr, self.col_idx, self.val = row_ptr, col_idx, val
        self.shape = (row_ptr.shape[0] - 1, row_ptr.shape[0] - 1)

    def __matmul__(self, X):
        if X.ndim == 1:
            return spmm(self.row_ptr, self.col_idx, self.val, X[:, None])[:, 0]
        return spmm(self.row_ptr, self.col_idx, self.val, X)

    def matmul_into(self, X, out):
        """out = A X for C-contiguous float64 X and out (n x m), no allocation."""
        assert X.flags.c_contiguous and out.flags.c_contiguous and X.shape == out.shape
        lib().orc_crs_spmm(self.shape[0], self.row_ptr, self.col_idx, self.val, X.shape[1], X.reshape(-1),
                           out.reshape(-1))


def pcg(row_ptr, col_idx, val, b, tol=1e-12, maxit=200000, x0=None):
    """FP64 oracle solve to the true relative residual tol -> (x, rc, iters, relres)."""
    n = b.shape[0]
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(0)
    rr = C.c_double(0)
    rc = lib().orc_pcg(n, row_ptr, col_idx, val, x, np.ascontiguousarray(b, dtype=np.float64), maxit, tol,
                       C.byref(it), C.byref(rr))
    return x, rc, it.value, rr.value


def reduce_crs(row_ptr, col_idx, val, remove_ids):
    """reduce_crs_matrix (LinearSolverClass.f90:3824-3947)."""
    n = row_ptr.shape[0] - 1
    rem = np.ascontiguousarray(remove_ids, dtype=np.int32)
    nnz = lib().orc_reduce_crs(n, row_ptr, col_idx, val, rem.shape[0], rem, None, None, None)
    nrow = n - np.unique(rem[(rem >= 1) & (rem <= n)]).shape[0]
    rp = np.zeros(nrow + 1, dtype=np.int64)
    ci = np.zeros(nnz, dtype=np.int32)
    v = np.zeros(nnz)
    lib().orc_reduce_crs(n, row_ptr, col_idx, val, rem.shape[0], rem, rp.ctypes.data, ci.ctypes.data,
                         v.ctypes.data)
    return rp, ci, v


def crs_to_scipy(row_ptr, col_idx, val, n=None):
    import scipy.sparse as sp
    n = row_ptr.shape[0] - 1 if n is None else n
    return sp.csr_matrix((val, col_idx.astype(np.int64) - 1, row_ptr - 1), shape=(n, n))

"""ctypes binding of libpfg.so (include/pfg.h).

The library is built in-tree by ``plantfem_gb300/build.py``.  There is no
fallback: if the shared library is missing or cannot be loaded, every call
raises ``NativeError`` -- the solve path only exists on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpfg.so")

PFG_OK = 0
PFG_W_NOT_CONVERGED = 1
ERRORS = {
    -1: "PFG_E_ARG", -2: "PFG_E_STATE", -3: "PFG_E_MISSING_SLOT", -4: "PFG_E_BREAKDOWN", -5: "PFG_E_NOMEM",
    -6: "PFG_E_CUDA", -7: "PFG_E_DETJ", -8: "PFG_E_INTERNAL", -9: "PFG_E_UNSUPPORTED", -10: "PFG_E_NONFINITE",
    -11: "PFG_E_ABORTED",
}

ALG_BICGSTAB, ALG_CG = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
STORAGE_FULL, STORAGE_SYMMETRIC = 0, 1
PC_NONE, PC_JACOBI, PC_BLOCK_JACOBI = 0, 1, 2
PC_ILU0, PC_ILU0_SORTED = 3, 4  # ILU(0): stored / ascending column order
STOP_REFERENCE, STOP_TRUE_RELATIVE = 0, 1


class NativeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SolveOpts(C.Structure):
    _fields_ = [("algorithm", C.c_int32), ("precision", C.c_int32), ("precond", C.c_int32),
                ("stop_rule", C.c_int32), ("itrmax", C.c_int32), ("graph_chunk", C.c_int32),
                ("er0", C.c_double), ("relative_er", C.c_double), ("reliable_delta", C.c_double),
                ("debug", C.c_int32), ("update_mode", C.c_int32), ("storage", C.c_int32)]


class EigOpts(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("max_itr", C.c_int32), ("tol", C.c_double), ("precision", C.c_int32),
                ("precond", C.c_int32), ("stop_rule", C.c_int32), ("debug", C.c_int32), ("seed", C.c_uint64),
                ("tol_fp32", C.c_double)]


EIG_STOP_REFERENCE, EIG_STOP_RESIDUAL = 0, 1


class NewmarkParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("newmark_beta", C.c_double), ("newmark_gamma", C.c_double),
                ("rayleigh_alpha", C.c_double), ("rayleigh_beta", C.c_double)]


class BatchConfig(C.Structure):
    _fields_ = [("threads", C.c_int32), ("cluster", C.c_int32), ("team_fraction", C.c_double)]

    def as_dict(self) -> dict:
        return {"threads": self.threads, "cluster": self.cluster, "team_fraction": self.team_fraction}


class BatchInfo(C.Structure):
    _fields_ = [("config", BatchConfig), ("launches", C.c_int32), ("max_iterations", C.c_int32),
                ("total_iterations", C.c_int64), ("max_rel_residual", C.c_double), ("solve_ms", C.c_double),
                ("fallbacks", C.c_int32)]

    def as_dict(self) -> dict:
        return {"config": self.config.as_dict(), "launches": self.launches, "max_iterations": self.max_iterations,
                "total_iterations": self.total_iterations, "max_rel_residual": self.max_rel_residual,
                "solve_ms": self.solve_ms, "fallbacks": self.fallbacks}


class Info(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("replacements", C.c_int32),
                ("kernel_launches", C.c_int32), ("rel_residual", C.c_double), ("iter_residual", C.c_double),
                ("solve_ms", C.c_double), ("fallback", C.c_int32)]

    def as_dict(self) -> dict:
        return {"status": self.status, "iterations": self.iterations, "replacements": self.replacements,
                "kernel_launches": self.kernel_launches, "rel_residual": self.rel_residual,
                "iter_residual": self.iter_residual, "solve_ms": self.solve_ms, "fallback": self.fallback}


_P = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_d = C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "pfg_solve_opts_default": (None, [C.POINTER(SolveOpts)]),
    "pfg_last_error": (C.c_char_p, []),
    "pfg_version": (C.c_char_p, []),
    "pfg_create": (C.c_int, [C.POINTER(_P)]),
    "pfg_destroy": (C.c_int, [_P]),
    "pfg_set_mesh": (C.c_int, [_P, _i64, _P, _i64, _i32, _P]),
    "pfg_set_crs": (C.c_int, [_P, _i32]),
    "pfg_set_crs_arrays": (C.c_int, [_P, _i64, _P, _P, _P]),
    "pfg_get_crs_size": (C.c_int, [_P, C.POINTER(_i64), C.POINTER(_i64)]),
    "pfg_get_crs": (C.c_int, [_P, _P, _P, _P]),
    "pfg_set_rhs": (C.c_int, [_P, _i64, _P]),
    "pfg_get_rhs": (C.c_int, [_P, _i64, _P]),
    "pfg_set_matrix": (C.c_int, [_P, _i32, _i32, _i32, _P]),
    "pfg_set_matrices": (C.c_int, [_P, _i64, _P, _P]),
    "pfg_set_vector": (C.c_int, [_P, _i32, _i32, _i32, _P]),
    "pfg_assemble_stiffness": (C.c_int, [_P, _i64, _P, _P]),
    "pfg_assemble_mass": (C.c_int, [_P, _i64, _P, _i32]),
    "pfg_assemble_body_force": (C.c_int, [_P, _i64, _P, _P]),
    "pfg_zeros": (C.c_int, [_P]),
    "pfg_fix": (C.c_int, [_P, _i64, _P, _P, _d]),
    "pfg_solve": (C.c_int, [_P, C.POINTER(SolveOpts), _P, _P, C.POINTER(Info)]),
    "pfg_crs_spmv_real64": (C.c_int, [_P, _P, _P, _P, _P, C.c_size_t, C.c_size_t]),
    "pfg_crs_spmv_real32": (C.c_int, [_P, _P, _P, _P, _P, C.c_size_t, C.c_size_t]),
    "pfg_linear_solver_crs": (C.c_int, [_P, _P, _P, _P, _P, _i64, _i64, C.POINTER(SolveOpts), C.POINTER(Info)]),
    "pfg_dev_spmv": (C.c_int, [_P, _P, _P, _P]),
    "pfg_dev_solve": (C.c_int, [_P, C.POINTER(SolveOpts), _P, _P, C.POINTER(Info), _P]),
    "pfg_profile_kernel": (C.c_int, [_P, _i32, _i32, C.POINTER(_d), C.POINTER(_d)]),
    "pfg_keep_this_matrix_as": (C.c_int, [_P, C.c_char_p]),
    "pfg_fix_eig": (C.c_int, [_P, _i64, _P]),
    "pfg_load_matrix": (C.c_int, [_P, C.c_char_p]),
    "pfg_eig_opts_default": (None, [C.POINTER(EigOpts)]),
    "pfg_eig": (C.c_int, [_P, C.POINTER(EigOpts), _i32, _P, _P, C.POINTER(Info)]),
    "pfg_eig_dense": (C.c_int, [_P, _i32, _P, _P, C.POINTER(Info)]),
    "pfg_eig_reduced_size": (C.c_int, [_P, C.POINTER(_i64)]),
    "pfg_linear_solver_crs_noalloc": (C.c_int, [_P, _P, _P, _P, _P, _i64, C.POINTER(SolveOpts), C.POINTER(Info),
                                                _P]),
    "pfg_eliminate": (C.c_int, [_P]),
    "pfg_ilu_reset": (C.c_int, [_P]),
    "pfg_ilu_factor": (C.c_int, [_P, C.c_int32, _P]),
    "pfg_ilu_apply": (C.c_int, [_P, _P, _P]),
    "pfg_ilu_solve": (C.c_int, [_P, _P, _P]),
    "pfg_element_stress": (C.c_int, [_P, _P, _i64, _P, _P, _i32, _P]),
    "pfg_dev_assemble_stiffness": (C.c_int, [_P, _i64, _P, _P, _P]),
    "pfg_dev_set_rhs": (C.c_int, [_P, _i64, _P, _P]),
    "pfg_dev_adjoint_grad_E": (C.c_int, [_P, _P, _P, _i64, _P, _P, _P]),
    "pfg_newmark_params_default": (None, [C.POINTER(NewmarkParams)]),
    "pfg_newmark_setup": (C.c_int, [_P, C.POINTER(NewmarkParams)]),
    "pfg_newmark_set_state": (C.c_int, [_P, _i64, _P, _P, _P]),
    "pfg_newmark_step": (C.c_int, [_P, C.POINTER(SolveOpts), _i64, _P, _P, _P, _P, C.POINTER(Info)]),
    "pfg_batch_create": (C.c_int, [C.POINTER(_P)]),
    "pfg_batch_destroy": (C.c_int, [_P]),
    "pfg_batch_set": (C.c_int, [_P, _i64, _P]),
    "pfg_batch_solve": (C.c_int, [_P, C.POINTER(SolveOpts), _P, _P, C.POINTER(BatchInfo)]),
    "pfg_batch_get_x": (C.c_int, [_P, _i64, _P]),
    "pfg_batch_set_config": (C.c_int, [_P, C.POINTER(BatchConfig)]),
    "pfg_batch_get_config": (C.c_int, [_P, C.POINTER(BatchConfig), C.POINTER(_i32)]),
    "pfg_batch_tune": (C.c_int, [_P, C.POINTER(SolveOpts), C.POINTER(BatchConfig), C.POINTER(_d)]),
    "pfg_batch_abort_flag": (C.c_int, [_P, C.POINTER(C.POINTER(_i32))]),
}

_LIB = None


def load():
    """Load libpfg.so; raise if it is absent (no CPU fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise NativeError(-9, f"{LIB_PATH} is not built; run plantfem_gb300/build.py "
                              "(the solve path has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def check(rc: int, allow_warning: bool = True) -> int:
    if rc == PFG_OK or (allow_warning and rc > 0):
        return rc
    msg = load().pfg_last_error().decode(errors="replace")
    raise NativeError(rc, msg)


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    load().pfg_solve_opts_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def ptr(a) -> int:
    """Address of a numpy array's data (C-contiguous required) or a torch tensor."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data

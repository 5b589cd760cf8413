"""pfg_linear_solver_crs_noalloc: the CG solve that allocates nothing.

Some callers cannot allocate device memory (their GPU memory belongs to
another runtime or a fixed pool, or they must not let cudaMalloc/cudaFree
synchronise the device while other work is queued).  For them the library
keeps the solver's work vectors in one static device array and takes the CRS
system in device memory.  This test calls that entry point through the C ABI
twice in a row and checks both results against the allocating plug-in
pfg_linear_solver_crs on the same system, within the 1e-8 relative tolerance
the other solve tests use.  It lives in its own file, named to be collected
last, and passes both alone and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from plantfem_gb300 import _native as N
from plantfem_gb300 import linear_solver_crs, problems

pytestmark = pytest.mark.gpu


def _system():
    p = problems.lognormal(9, seed=4)
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=p["E"], nu=p["nu"])
    b = p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    return rp, ci, val, b


def test_noalloc_matches_allocating_plugin_twice(cuda):
    import torch
    rp, ci, val, b = _system()
    n = b.shape[0]
    lib = N.load()
    opts = N.default_opts(algorithm=N.ALG_CG, precision=N.PREC_FP64, precond=N.PC_JACOBI,
                          stop_rule=N.STOP_TRUE_RELATIVE, relative_er=1e-12)
    # the allocating plug-in (host arrays) as the reference result
    x_ref = np.zeros(n)
    info = linear_solver_crs(rp, ci, val, b, x_ref, algorithm="CG", precision="fp64", preconditioning="Jacobi",
                             relative_er=1e-12)
    assert info["status"] == 0
    # device inputs and outputs; the entry point itself allocates nothing
    d_rp = torch.from_numpy(rp).to(cuda)
    d_ci = torch.from_numpy(ci).to(cuda)
    d_val = torch.from_numpy(val).to(cuda)
    d_b = torch.from_numpy(b).to(cuda)
    torch.cuda.synchronize()
    for call in range(2):
        d_x = torch.zeros(n, dtype=torch.float64, device=cuda)
        torch.cuda.synchronize()
        inf = N.Info()
        rc = lib.pfg_linear_solver_crs_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), d_val.data_ptr(), d_b.data_ptr(),
                                               d_x.data_ptr(), n, C.byref(opts), C.byref(inf), None)
        assert rc == 0, lib.pfg_last_error()
        assert inf.status == 0 and inf.rel_residual <= 1e-12, inf.as_dict()
        x = d_x.cpu().numpy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e-8, call


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    lib = N.load()
    n = 262145
    rc = lib.pfg_linear_solver_crs_noalloc(1, 1, 1, 1, 1, n, None, None, None)  # checked before any access
    assert rc == -1
    assert b"exceeds the static scratch limit" in lib.pfg_last_error()

"""pfg_linear_solver_crs_noalloc: the CG solve that allocates nothing.

Some callers cannot allocate device memory: their GPU memory belongs to
another runtime or to a fixed-size pool, or they must not let cudaMalloc /
cudaFree synchronise the device while other work is queued.  For them the
library keeps the solver's work vectors in one static device array and takes
the CRS system in device memory.

These tests call that entry point through the C ABI and check it against the
FP64 oracle (Jacobi CG to the true relative residual 1e-12) and against the
allocating plug-in pfg_linear_solver_crs, within the 1e-8 relative tolerance
the other solve tests use, on two calls in a row; at a size just under the
static limit; that a solve after the set-up call leaves the device's free
memory unchanged; and the NULL-options, no-preconditioner, unsupported-option
and not-converged paths.  The file is named to be collected last and passes
both alone and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from plantfem_gb300 import _native as N
from plantfem_gb300 import linear_solver_crs, problems

pytestmark = pytest.mark.gpu

MAX_DOF = 262144  # the static scratch limit stated in include/pfg.h
TOL = 1e-8        # relative displacement tolerance of the solve tests


def _stiffness_system():
    p = problems.lognormal(9, seed=4)
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=p["E"], nu=p["nu"])
    b = p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    return rp, ci, val, b


def _near_limit_system():
    """Consistent mass matrix of a 43^3 cube: 255,552 DOF, just under the limit.

    The mass matrix is symmetric positive definite and well conditioned, so the
    oracle's CG reaches 1e-12 in under a hundred iterations.
    """
    nc, en = O.cube3d(43, 43, 43)
    rp, ci = O.zero_matrix(nc.shape[0], en, 3)
    val = O.assemble(nc, en, rp, ci, "mass", rho=np.full(en.shape[0], 1.0e3))
    b = np.random.default_rng(7).standard_normal(rp.shape[0] - 1)
    return rp, ci, val, b


def _to_device(cuda, *arrays):
    import torch
    out = [torch.from_numpy(a).to(cuda) for a in arrays]
    torch.cuda.synchronize()
    return out


def _solve(lib, dev, n, opts, x0=None):
    """One call through the C ABI; returns (rc, info, x on the host)."""
    import torch
    d_rp, d_ci, d_val, d_b = dev
    d_x = torch.zeros(n, dtype=torch.float64, device=d_b.device) if x0 is None else x0
    torch.cuda.synchronize()
    inf = N.Info()
    rc = lib.pfg_linear_solver_crs_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), d_val.data_ptr(), d_b.data_ptr(),
                                           d_x.data_ptr(), n, None if opts is None else C.byref(opts),
                                           C.byref(inf), None)
    return rc, inf, d_x.cpu().numpy()


def _rel(x, ref):
    return np.linalg.norm(x - ref) / np.linalg.norm(ref)


def _opts(**kw):
    base = dict(algorithm=N.ALG_CG, precision=N.PREC_FP64, precond=N.PC_JACOBI,
                stop_rule=N.STOP_TRUE_RELATIVE, relative_er=1e-12)
    base.update(kw)
    return N.default_opts(**base)


def test_noalloc_matches_oracle_and_allocating_plugin_twice(cuda):
    rp, ci, val, b = _stiffness_system()
    n = b.shape[0]
    lib = N.load()
    x_orc = O.pcg(rp, ci, val, b, tol=1e-12)[0]
    x_plug = np.zeros(n)
    info = linear_solver_crs(rp, ci, val, b, x_plug, algorithm="CG", precision="fp64", preconditioning="Jacobi",
                             relative_er=1e-12)
    assert info["status"] == 0
    dev = _to_device(cuda, rp, ci, val, b)
    for call in range(2):
        rc, inf, x = _solve(lib, dev, n, _opts())
        assert rc == 0, lib.pfg_last_error()
        assert inf.status == 0 and inf.rel_residual <= 1e-12, inf.as_dict()
        assert _rel(x, x_orc) <= TOL, (call, _rel(x, x_orc))
        assert _rel(x, x_plug) <= TOL, (call, _rel(x, x_plug))


def test_noalloc_near_its_limit_matches_oracle_twice(cuda):
    rp, ci, val, b = _near_limit_system()
    n = b.shape[0]
    assert MAX_DOF - 10000 < n <= MAX_DOF
    lib = N.load()
    x_orc = O.pcg(rp, ci, val, b, tol=1e-12)[0]
    dev = _to_device(cuda, rp, ci, val, b)
    for call in range(2):
        rc, inf, x = _solve(lib, dev, n, _opts())
        assert rc == 0, lib.pfg_last_error()
        assert inf.status == 0, inf.as_dict()
        assert _rel(x, x_orc) <= TOL, (call, _rel(x, x_orc))


def test_noalloc_solve_leaves_free_device_memory_unchanged(cuda):
    import torch
    rp, ci, val, b = _stiffness_system()
    n = b.shape[0]
    lib = N.load()
    assert lib.pfg_linear_solver_crs_noalloc(None, None, None, None, None, 0, None, None, None) == 0, \
        lib.pfg_last_error()
    dev = _to_device(cuda, rp, ci, val, b)
    x0 = torch.zeros(n, dtype=torch.float64, device=cuda)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc, inf, _ = _solve(lib, dev, n, _opts(), x0=x0)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert rc == 0, lib.pfg_last_error()
    assert free_after == free_before, (free_before, free_after)


def test_noalloc_default_options_and_no_preconditioner(cuda):
    rp, ci, val, b = _stiffness_system()
    n = b.shape[0]
    lib = N.load()
    x_orc = O.pcg(rp, ci, val, b, tol=1e-12)[0]
    dev = _to_device(cuda, rp, ci, val, b)
    # opts NULL: CG + point Jacobi to the true relative residual 1e-10
    rc, inf, x = _solve(lib, dev, n, None)
    assert rc == 0, lib.pfg_last_error()
    assert inf.status == 0 and inf.rel_residual <= 1e-10, inf.as_dict()
    assert _rel(x, x_orc) <= 1e-6
    rc, inf, x = _solve(lib, dev, n, _opts(precond=N.PC_NONE))
    assert rc == 0, lib.pfg_last_error()
    assert _rel(x, x_orc) <= TOL


def test_noalloc_reports_not_converged_and_rejects_other_options(cuda):
    rp, ci, val, b = _stiffness_system()
    n = b.shape[0]
    lib = N.load()
    dev = _to_device(cuda, rp, ci, val, b)
    rc, inf, x = _solve(lib, dev, n, _opts(itrmax=5))
    assert rc == N.PFG_W_NOT_CONVERGED and inf.status == N.PFG_W_NOT_CONVERGED
    assert inf.iterations == 5 and np.all(np.isfinite(x))
    for bad in (dict(stop_rule=N.STOP_REFERENCE), dict(algorithm=N.ALG_BICGSTAB), dict(precision=N.PREC_MIXED),
                dict(precond=N.PC_BLOCK_JACOBI)):
        rc, _, _ = _solve(lib, dev, n, _opts(**bad))
        assert rc == -9, (bad, lib.pfg_last_error())  # PFG_E_UNSUPPORTED


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    lib = N.load()
    rc = lib.pfg_linear_solver_crs_noalloc(1, 1, 1, 1, 1, MAX_DOF + 1, None, None, None)  # checked before any access
    assert rc == -1
    assert b"exceeds the static scratch limit" in lib.pfg_last_error()

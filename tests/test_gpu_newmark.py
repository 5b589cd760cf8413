"""Linear Newmark-beta time stepping (SeismicAnalysis_%LinearReyleighNewmark).

A small cantilever under a gravity-like external acceleration is stepped on
the GPU and by the oracle: the oracle assembles K and the consistent M on the
CPU, forms the reference's right-hand side literally with its a(1..8)
coefficients (SeismicAnalysisClass.f90:1478-1499) and C = alpha M + beta K,
eliminates the fixed DOFs as LinearSolver_%fix does, solves directly (SuperLU)
and updates v and a with updateVelocity/AccelNewmarkBeta (:1501-1535).  U, V
and A agree to 1e-8 (relative, per step) over 6 steps.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

import oracle as O
from plantfem_gb300 import FEMDomain, SeismicAnalysis

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _oracle_steps(dom, rho, E, nu, fixed_ids, a_ext, dt, b, g, al, be, steps):
    nn, ne = dom.nn(), dom.ne()
    rp, ci = O.zero_matrix(nn, dom.elemnod, 3)
    Kv = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=E, nu=nu)
    Mv = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "mass", rho=rho)
    K = O.crs_to_scipy(rp, ci, Kv)
    M = O.crs_to_scipy(rp, ci, Mv)
    C = al * M + be * K
    Aeff_v = (1.0 / (b * dt * dt)) * Mv + (g / (b * dt)) * (al * Mv + be * Kv) + Kv
    n = 3 * nn
    fixed = np.zeros(n, np.uint8)
    fixed[fixed_ids - 1] = 1
    base = np.zeros(n)
    Ae = Aeff_v.copy()
    O.apply_fix(rp, ci, Ae, base, fixed, np.zeros(n))
    A_e = O.crs_to_scipy(rp, ci, Ae).tocsc()
    a = np.zeros(9)
    a[1] = g / (b * dt)
    a[2] = -g / (b * dt)
    a[3] = 1.0 - g / b
    a[4] = dt * (1.0 - g / (2.0 * b))
    a[5] = 1.0 / (b * dt * dt)
    a[6] = -1.0 / (b * dt * dt)
    a[7] = -1.0 / (b * dt)
    a[8] = 1.0 - 1.0 / (2.0 * b)
    u, v, acc = np.zeros(n), np.zeros(n), np.zeros(n)
    out = []
    for _ in range(steps):
        force = M @ a_ext
        R = (force - a[6] * (M @ u) - a[7] * (M @ v) - a[8] * (M @ acc)
             - a[2] * (C @ u) - a[3] * (C @ v) - a[4] * (C @ acc))
        rhs = np.where(fixed == 1, base, R + base)
        un = sla.spsolve(A_e, rhs)
        vn = g / (b * dt) * un - g / (b * dt) * u + (1.0 - g / b) * v + dt * (1.0 - g / (2.0 * b)) * acc
        an = un / (b * dt * dt) - u / (b * dt * dt) - v / (b * dt) + (1.0 - 1.0 / (2.0 * b)) * acc
        u, v, acc = un, vn, an
        out.append((u.copy(), v.copy(), acc.copy()))
    return out


@pytest.mark.parametrize("precision,storage", [("fp64", "full"), ("mixed", "symmetric")])
def test_newmark_matches_oracle(cuda, precision, storage):
    dom = FEMDomain().create("Cube3D", 3, 3, 6)
    ne, nn = dom.ne(), dom.nn()
    rho, E, nu = 1000.0, 1.0e6, 0.3
    sa = SeismicAnalysis().init(dom, rho, E, nu)
    sa.dt = 1.0e-3
    base_nodes = np.nonzero(dom.nodcoord[:, 2] <= 0.0)[0] + 1
    for d in "xyz":
        sa.fixDisplacement(base_nodes, d, 0.0)
    a_ext = np.zeros(3 * nn)
    a_ext[2::3] = -9.8
    sa.A_ext = a_ext
    fixed_ids = np.sort(np.concatenate([3 * (base_nodes - 1) + k + 1 for k in range(3)]))
    ref = _oracle_steps(dom, np.full(ne, rho), np.full(ne, E), np.full(ne, nu), fixed_ids, a_ext, sa.dt,
                        sa.Newmark_beta, sa.Newmark_gamma, sa.alpha, sa.beta, 6)
    for k, (ur, vr, ar) in enumerate(ref):
        sa.LinearReyleighNewmark(TOL=1e-12, precision=precision, storage=storage)
        assert sa.last_info["status"] == 0, sa.last_info
        assert _rel(sa.U, ur) <= 1e-8, (k, _rel(sa.U, ur))
        assert _rel(sa.V, vr) <= 1e-8, (k, _rel(sa.V, vr))
        assert _rel(sa.A, ar) <= 1e-7, (k, _rel(sa.A, ar))
        assert np.all(sa.U[fixed_ids - 1] == 0.0)


def test_newmark_setup_needs_kept_matrices(cuda):
    import ctypes as C
    from plantfem_gb300 import FEMSolver
    from plantfem_gb300 import _native as N
    dom = FEMDomain().create("Cube3D", 2, 2, 2)
    s = FEMSolver()
    s.setDomain(dom)
    s.setCRS(3)
    p = N.NewmarkParams()
    N.load().pfg_newmark_params_default(C.byref(p))
    assert p.newmark_beta == 0.25 and p.newmark_gamma == 0.5 and p.rayleigh_alpha == 0.524
    assert N.load().pfg_newmark_setup(s.handle, C.byref(p)) == -2  # no "A"/"B" kept
    n = 3 * dom.nn()
    assert N.load().pfg_newmark_step(s.handle, None, n, None, None, None, None, None) == -2  # no set-up

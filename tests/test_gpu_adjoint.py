"""Adjoint dL/dE (the differentiation form) and stress recovery on the GPU.

dL/dE from one adjoint solve is checked against (1) a reference gradient built
entirely from FP64 oracle solves on the CPU, (2) central finite differences
(h = 1e-4 E_e) of the GPU forward solve.  Tolerances: 1e-7 relative to the
largest gradient entry against the oracle gradient (two 1e-12 solves);
1e-5 against central differences (O(h^2) truncation plus solve noise).
"""
import numpy as np
import pytest
import torch

import oracle as O
from plantfem_gb300 import FEMDomain, FEMSolver, problems
from plantfem_gb300.adjoint import ElasticOperator

pytestmark = pytest.mark.gpu


def _problem(n=6):
    p = problems.lognormal(n, seed=11)
    E_true = problems.lognormal_E(p["domain"].ne(), seed=1)
    E = problems.lognormal_E(p["domain"].ne(), seed=2)
    return p, E_true, E


def _oracle_grad(p, E, u_t):
    dom = p["domain"]
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    val = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=E, nu=p["nu"])
    b = p["rhs"].copy()
    fixed = np.zeros(3 * dom.nn(), np.uint8)
    fixed[p["fix_ids"] - 1] = 1
    O.apply_fix(rp, ci, val, b, fixed, np.zeros(3 * dom.nn()))
    u, rc, _, _ = O.pcg(rp, ci, val, b, tol=1e-13)
    g = u - u_t
    g[fixed == 1] = 0.0
    lam, rc2, _, _ = O.pcg(rp, ci, val, g, tol=1e-13)
    assert rc == 0 and rc2 == 0
    Kh = O.element_stiffness_all(dom.nodcoord, dom.elemnod, 1.0, p["nu"])
    en = dom.elemnod - 1
    dofs = (3 * en[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 24)
    return -np.einsum("ei,eij,ej->e", lam[dofs], Kh, u[dofs]), u


@pytest.mark.parametrize("precision,recompute", [("fp64", False), ("fp64", True), ("mixed", False)])
def test_adjoint_gradient_vs_oracle_and_fd(cuda, precision, recompute):
    p, E_true, E = _problem()
    op = ElasticOperator(p["domain"], p["nu"], p["rhs"], p["fix_ids"], precision=precision, relative_er=1e-12,
                         recompute_u=recompute)
    u_t = op.displacement(torch.tensor(E_true, device=cuda)).detach()
    Et = torch.tensor(E, device=cuda, requires_grad=True)
    u = op.displacement(Et)
    L = 0.5 * torch.sum((u - u_t) ** 2)
    L.backward()
    g = Et.grad.cpu().numpy()
    g_ref, _ = _oracle_grad(p, E, u_t.cpu().numpy())
    assert np.abs(g - g_ref).max() <= 1e-7 * np.abs(g_ref).max()
    if precision == "fp64" and not recompute:
        rng = np.random.default_rng(3)
        for k in rng.choice(E.shape[0], size=8, replace=False):
            h = 1e-4 * E[k]
            Lp, Lm = [], []
            for sgn, out in ((1, Lp), (-1, Lm)):
                Ek = E.copy()
                Ek[k] += sgn * h
                with torch.no_grad():
                    uk = op.displacement(torch.tensor(Ek, device=cuda))
                out.append(0.5 * float(torch.sum((uk - u_t) ** 2)))
            fd = (Lp[0] - Lm[0]) / (2 * h)
            assert abs(fd - g[k]) <= 1e-5 * np.abs(g).max(), (k, fd, g[k])


def test_element_stress_vs_oracle(cuda):
    dom = FEMDomain().create("Cube3D", 4, 3, 3)
    rng = np.random.default_rng(0)
    disp = rng.standard_normal(3 * dom.nn()) * 1e-3
    E = rng.uniform(1e3, 1e4, dom.ne())
    nu = rng.uniform(0.1, 0.4, dom.ne())
    s = FEMSolver()
    s.setDomain(dom)
    S = s.getElementCauchyStress(disp, E, nu)
    ref = O.element_stress(dom.nodcoord, dom.elemnod, disp, E, nu)
    assert np.abs(S - ref).max() <= 1e-12 * np.abs(ref).max()
    I1 = s.getElementCauchyStress(disp, E, nu, option="I1")
    np.testing.assert_allclose(I1, np.trace(ref, axis1=1, axis2=2), rtol=0, atol=1e-12 * np.abs(ref).max())


def _invariants(S):
    """The reference's formulas of getElementCauchyStress (FEMDomainClass.f90:15310-15362)."""
    tr = np.trace(S, axis1=1, axis2=2)
    I2 = 0.5 * (tr * tr - np.einsum("eij,eji->e", S, S))
    I3 = np.linalg.det(S)
    s = S - (tr / 3.0)[:, None, None] * np.eye(3)[None]
    trs = np.trace(s, axis1=1, axis2=2)
    J2 = 0.5 * (trs * trs - np.einsum("eij,eji->e", s, s))
    return {"p": tr / 3.0, "I1": tr, "I2": I2, "I3": I3, "J1": trs, "J2": J2, "J3": np.linalg.det(s)}


def test_element_stress_every_option_vs_oracle(cuda):
    """Every option string of getElementCauchyStress and the (i, j) form,
    computed on the GPU from the cell-averaged tensors, against the same
    formulas on the oracle's tensors; an unknown option gives zeros."""
    dom = FEMDomain().create("Cube3D", 4, 3, 3)
    rng = np.random.default_rng(3)
    disp = rng.standard_normal(3 * dom.nn()) * 1e-3
    E = rng.uniform(1e3, 1e4, dom.ne())
    nu = rng.uniform(0.1, 0.4, dom.ne())
    s = FEMSolver()
    s.setDomain(dom)
    ref = O.element_stress(dom.nodcoord, dom.elemnod, disp, E, nu)
    inv = _invariants(ref)
    scale = np.abs(ref).max()
    names = {"p": ["p", "P"], "I1": ["I", "I1", "i1", "trace", "tr", "TRACE", "TR"], "I2": ["II", "I2", "i2", "ii"],
             "I3": ["III", "I3", "i3", "iii"], "J1": ["J", "J1", "j1", "j"], "J2": ["JJ", "J2", "j2", "jj"],
             "J3": ["JJJ", "J3", "j3", "jjj"]}
    for key, opts in names.items():
        tol = 1e-12 * (scale ** (3 if key in ("I3", "J3") else 2 if key in ("I2", "J2") else 1))
        for o in opts:
            got = s.getElementCauchyStress(disp, E, nu, option=o)
            assert np.abs(got - inv[key]).max() <= tol, (o, np.abs(got - inv[key]).max())
    comps = {"1,1": (0, 0), "2,2": (1, 1), "3,3": (2, 2), "1,2": (0, 1), "2,1": (0, 1), "1,3": (0, 2),
             "3,1": (0, 2), "3,2": (1, 2), "2,3": (1, 2)}
    for o, (a, b) in comps.items():
        for form in (o, f"({o})", "_{" + o + "}"):
            got = s.getElementCauchyStress(disp, E, nu, option=form)
            assert np.abs(got - ref[:, a, b]).max() <= 1e-12 * scale, form
    for a in range(3):
        for b in range(3):
            got = s.getElementCauchyStress(disp, E, nu, i=a + 1, j=b + 1)
            assert np.abs(got - ref[:, a, b]).max() <= 1e-12 * scale, (a, b)
    assert np.array_equal(s.getElementCauchyStress(disp, E, nu, option="von Mises"), np.zeros(dom.ne()))


def test_gravity_bar_stress_kat_gpu(cuda):
    """benchmark_bar_in_gravity_field.f90:56-67 end to end on the GPU:
    I1 of element 1 = -234.026 on the deformed mesh (theory -234.024), with the
    stress recovered by the GPU element kernel."""
    dom = FEMDomain().create("Cube3D", 10, 10, 100)
    dom.resize(z=10.0)
    s = FEMSolver()
    s.setDomain(dom)
    s.setCRS(3)
    s.assembleStiffness(2.17e7, 0.0)
    s.assembleBodyForce(2.4, [0.0, 0.0, -9.8])
    for d in (2, 1, 0):
        s.fix(1, dom.select(z_max=dom.z_min()) * 3 - d, FixValue=0.0)
    x = s.solve()
    I1_undeformed = s.getElementCauchyStress(x, [2.17e7], [0.0], option="I1")[0]
    ref = O.element_stress(dom.nodcoord, dom.elemnod, x, 2.17e7, 0.0)
    assert abs(I1_undeformed - np.trace(ref[0])) <= 1e-12 * abs(I1_undeformed)
    dom.deform(disp=x)
    t = FEMSolver()
    t.setDomain(dom)
    I1 = t.getElementCauchyStress(x, [2.17e7], [0.0], option="I1")[0]
    assert abs(I1 - (-234.026)) < 1e-3

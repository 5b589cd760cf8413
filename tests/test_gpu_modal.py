"""Modal analysis callers on the GPU against the FP64 oracle.

SeismicAnalysis_%modalAnalysis (SeismicAnalysisClass.f90:1715-1834) and
ModalAnalysis_%solve (ModalAnalysisClass.f90:115-179) assemble M and K, drop
the fixed nodes' DOFs and solve K x = lambda M x -- by default every pair by
the dense branch of FEMSolver_%eig.  The oracle: the oracle-assembled K and M,
reduced by reduce_crs_matrix, solved by LAPACK's generalized symmetric-definite
solver (scipy eigh type 1, the DSPGVD stand-in).  Bars: frequencies within
1e-9 relative (dense) and 1e-7 (LOBPCG); modes of well-separated frequencies
parallel to the oracle's to 1e-8; the reference's constants (3.141590 in
modalAnalysis, pi in ModalAnalysis) and mode normalisation.
"""
import math

import numpy as np
import pytest
import scipy.linalg as sla

import oracle as O
from plantfem_gb300 import FEMDomain, ModalAnalysis, SeismicAnalysis

pytestmark = pytest.mark.gpu


def _domain():
    # an irregular brick (4 x 3 x 2 elements of unequal sides, lognormal E):
    # no symmetry, so the modes are unique up to sign
    dom = FEMDomain().create("Cube3D", x_num=4, y_num=3, z_num=2, x_len=2.0, y_len=1.3, z_len=0.7)
    rng = np.random.default_rng(17)
    E = np.exp(rng.normal(np.log(1e4), 0.3, dom.ne()))
    rho = rng.uniform(800.0, 1200.0, dom.ne())
    return dom, E, rho


def _oracle(dom, E, nu, rho, fixed_dofs):
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    K = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "stiffness", E=E, nu=nu)
    M = O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "mass", rho=rho)
    ids = np.asarray(fixed_dofs, dtype=np.int32)
    rk, ck, vk = O.reduce_crs(rp, ci, K, ids)
    rm, cm, vm = O.reduce_crs(rp, ci, M, ids)
    w, Z = sla.eigh(O.crs_to_scipy(rk, ck, vk).toarray(), O.crs_to_scipy(rm, cm, vm).toarray(), type=1)
    keep = np.setdiff1d(np.arange(3 * dom.nn()), ids - 1)
    return w, Z, keep


def _x0_nodes(dom):
    return np.nonzero(dom.nodcoord[:, 0] <= 0.0)[0] + 1


def test_seismic_modal_analysis_dense_vs_oracle(cuda):
    dom, E, rho = _domain()
    nodes = _x0_nodes(dom)
    sa = SeismicAnalysis()
    freq, X = sa.modalAnalysis(dom, E, 0.3, rho, fix_node_list_x=nodes, fix_node_list_y=nodes,
                               fix_node_list_z=nodes)
    fixed = np.sort(np.concatenate([(nodes - 1) * 3 + d for d in (1, 2, 3)]))
    w, Z, keep = _oracle(dom, E, np.full(dom.ne(), 0.3), rho, fixed)
    f_ref = np.sqrt(np.abs(w)) / 2.0 / 3.141590
    assert freq.shape == f_ref.shape
    assert np.all(np.abs(freq - f_ref) <= 1e-9 * f_ref)
    assert np.array_equal(sa.frequency, freq)
    # unit 2-norm modes, zero at the fixed DOFs, parallel to the oracle's
    assert np.allclose(np.linalg.norm(X, axis=0), 1.0, rtol=0, atol=1e-12)
    assert np.abs(X[fixed - 1]).max() == 0.0
    gaps = np.minimum(np.diff(w, prepend=-np.inf), np.diff(w, append=np.inf)) / w
    for k in np.nonzero(gaps > 1e-3)[0][:20]:
        z = np.zeros(X.shape[0])
        z[keep] = Z[:, k]
        cos = abs(np.dot(X[:, k], z)) / np.linalg.norm(z)
        assert cos >= 1.0 - 1e-8, (k, cos)


def test_seismic_modal_analysis_lobpcg_option(cuda):
    dom, E, rho = _domain()
    nodes = _x0_nodes(dom)
    sa = SeismicAnalysis()
    freq, X = sa.modalAnalysis(dom, E, 0.3, rho, fix_node_list_x=nodes, fix_node_list_y=nodes,
                               fix_node_list_z=nodes, num_eigen=5, use_LOBPCG=True, block_size=8)
    fixed = np.sort(np.concatenate([(nodes - 1) * 3 + d for d in (1, 2, 3)]))
    w, _, _ = _oracle(dom, E, np.full(dom.ne(), 0.3), rho, fixed)
    f_ref = np.sqrt(np.abs(w[:5])) / 2.0 / 3.141590
    assert np.all(np.abs(freq - f_ref) <= 1e-7 * f_ref)
    assert X.shape == (3 * dom.nn(), 5)


def test_modal_analysis_class_vs_oracle(cuda):
    dom, _, _ = _domain()
    ma = ModalAnalysis().init([dom])
    ma.setMaterial(DomainID=1, Density=[1.0e3], YoungModulus=[1.0e4], PoissonRatio=[0.3])
    nodes = _x0_nodes(dom)
    ma.setBoundary(DomainID=1, NodeList=nodes)
    f = ma.solve()
    fixed = np.sort(np.concatenate([(nodes - 1) * 3 + d for d in (1, 2, 3)]))
    ne = dom.ne()
    w, _, _ = _oracle(dom, np.full(ne, 1e4), np.full(ne, 0.3), np.full(ne, 1e3), fixed)
    f_ref = np.sqrt(np.abs(w)) / 2.0 / math.pi
    assert np.all(np.abs(f - f_ref) <= 1e-9 * f_ref)
    # EigenMode as eig returns it: B-orthonormal, not rescaled
    rp, ci = O.zero_matrix(dom.nn(), dom.elemnod, 3)
    M = O.crs_to_scipy(rp, ci, O.assemble(dom.nodcoord, dom.elemnod, rp, ci, "mass", rho=np.full(ne, 1e3)))
    G = ma.EigenMode.T @ (M @ ma.EigenMode)
    assert np.abs(G - np.eye(G.shape[0])).max() <= 1e-9
    ma.remove()


def test_modal_analysis_only_matrix_and_one_domain(cuda):
    dom, _, _ = _domain()
    ma = ModalAnalysis().init(dom)
    ma.setMaterial(1, Density=1.0e3, YoungModulus=1.0e4, PoissonRatio=0.3)
    assert ma.solve(only_matrix=True) is None and ma.EigenFrequency is None
    with pytest.raises(NotImplementedError):
        ModalAnalysis().init([dom, dom])
    ma.remove()

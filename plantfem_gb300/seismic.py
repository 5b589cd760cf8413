"""SeismicAnalysis: modal analysis and linear Newmark-beta time stepping.

Mirrors the fields and the step of plantFEM's ``SeismicAnalysis_``
(SeismicAnalysisClass.f90: defaults :98-109, ``LinearReyleighNewmark``
:1255-1436, Newmark formulas :1464-1535) over the GPU path: the stiffness and
consistent mass are assembled once on the device, combined into the Newmark
matrix, and every call of :meth:`LinearReyleighNewmark` advances one time step
(two SpMVs, one warm-started solve and the velocity/acceleration update on the
GPU; ``pfg_newmark_*`` in include/pfg.h).  The reference re-integrates every
element matrix at every step; the results are the same linear algebra.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .femdomain import FEMDomain
from .femsolver import FEMSolver


def _pinned(n):
    """(float64 array of n zeros in page-locked host memory, its owner); plain
    host memory when no CUDA device is visible."""
    try:
        import torch
        if torch.cuda.is_available():
            t = torch.zeros(n, dtype=torch.float64).pin_memory()
            return t.numpy(), t
    except Exception:
        pass
    return np.zeros(n), None


class SeismicAnalysis:
    # SeismicAnalysis_ public parameters (SeismicAnalysisClass.f90:98-109)
    dt: float = 1.0
    alpha: float = 0.524      # Rayleigh damping C = alpha M + beta K
    beta: float = 0.00129
    Newmark_beta: float = 0.25
    Newmark_gamma: float = 0.5

    def __init__(self):
        self.femdomain: FEMDomain | None = None
        self.Density = self.YoungModulus = self.PoissonRatio = None
        self.fixes: list[tuple[np.ndarray, np.ndarray]] = []
        self.U = self.V = self.A = self.A_ext = None
        self._s: FEMSolver | None = None
        self.last_info: dict = {}

    def init(self, femdomain: FEMDomain, Density, YoungModulus, PoissonRatio) -> "SeismicAnalysis":
        self.femdomain = femdomain
        ne = femdomain.ne()
        self.Density = np.broadcast_to(np.asarray(Density, dtype=np.float64), (ne,)).copy()
        self.YoungModulus = np.broadcast_to(np.asarray(YoungModulus, dtype=np.float64), (ne,)).copy()
        self.PoissonRatio = np.broadcast_to(np.asarray(PoissonRatio, dtype=np.float64), (ne,)).copy()
        n = 3 * femdomain.nn()
        # page-locked host arrays: every step copies A_ext in and U, V, A out
        # (on GB300 pageable copies took about a fifth of a 60^3 step)
        self._pins = [_pinned(n) for _ in range(4)]
        self.U, self.V, self.A, self.A_ext = (a for a, _ in self._pins)
        self._s = None
        return self

    # the reference's constant in the frequency of modalAnalysis
    # (SeismicAnalysisClass.f90:1805: freq = sqrt(|lambda|) / 2 / 3.141590)
    _PI_MODAL = 3.141590

    def modalAnalysis(self, femdomain: FEMDomain, YoungModulus, PoissonRatio, Density, fix_node_list_x=None,
                      fix_node_list_y=None, fix_node_list_z=None, num_eigen: int | None = None,
                      use_LOBPCG: bool = False, **eig_kw):
        """SeismicAnalysis_%modalAnalysis (SeismicAnalysisClass.f90:1715-1834).

        Assembles the consistent mass (kept as "B") and the stiffness (kept as
        "A") with per-element Density / YoungModulus / PoissonRatio, removes
        the listed nodes' x, y and z DOFs (1-based node ids -> DOF
        (id - 1) * 3 + d, fix_eig), solves the generalized eigenproblem --
        by default every pair with the dense branch, as the reference's
        ``eig()`` call does; ``use_LOBPCG`` (with ``num_eigen`` and
        ``eig_kw`` for FEMSolver.eig) for large meshes -- and sets
        ``frequency = sqrt(|lambda|) / 2 / 3.141590`` and ``ModeVectors``, each
        mode with a non-zero frequency scaled to unit 2-norm.
        Returns (frequency, ModeVectors).
        """
        ne = femdomain.ne()
        self.YoungModulus = np.broadcast_to(np.asarray(YoungModulus, dtype=np.float64), (ne,)).copy()
        self.PoissonRatio = np.broadcast_to(np.asarray(PoissonRatio, dtype=np.float64), (ne,)).copy()
        self.Density = np.broadcast_to(np.asarray(Density, dtype=np.float64), (ne,)).copy()
        self.femdomain = femdomain
        s = FEMSolver()
        s.setDomain(femdomain)
        s.setCRS(3)
        s.assembleMass(self.Density)
        s.keepThisMatrixAs("B")
        s.zeros()
        s.assembleStiffness(self.YoungModulus, self.PoissonRatio)
        s.keepThisMatrixAs("A")
        for d, lst in enumerate((fix_node_list_x, fix_node_list_y, fix_node_list_z)):
            if lst is not None and len(lst) > 0:
                s.fix_eig((np.asarray(lst, dtype=np.int64) - 1) * 3 + d + 1)
        s.use_LOBPCG = bool(use_LOBPCG)
        lam, X = s.eig(num_eigen, **eig_kw)
        freq = np.sqrt(np.abs(lam)) / 2.0 / self._PI_MODAL
        for i in range(freq.shape[0]):
            if freq[i] == 0.0:
                continue
            X[:, i] = X[:, i] / np.linalg.norm(X[:, i])
        self.frequency = freq
        self.ModeVectors = X
        self.last_info = dict(s.last_info)
        s.remove()
        return freq, X

    def fixDisplacement(self, NodeList, direction: str, disp: float = 0.0):
        """Prescribed displacement of nodes (1-based ids) in x, y or z
        (FixNodeList_x/y/z with FixNodeList_Disp_*)."""
        d = {"x": 0, "y": 1, "z": 2}[direction]
        ids = 3 * (np.asarray(NodeList, dtype=np.int64) - 1) + d + 1
        self.fixes.append((ids.astype(np.int32), np.full(ids.shape[0], float(disp))))
        self._s = None

    def _setup(self):
        s = FEMSolver()
        s.setDomain(self.femdomain)
        s.setCRS(3)
        s.assembleMass(self.Density)
        s.keepThisMatrixAs("B")
        s.zeros()
        s.assembleStiffness(self.YoungModulus, self.PoissonRatio)
        s.keepThisMatrixAs("A")
        for ids, vals in self.fixes:
            s.fix(1, ids, FixValues=vals)
        p = N.NewmarkParams(float(self.dt), float(self.Newmark_beta), float(self.Newmark_gamma), float(self.alpha),
                            float(self.beta))
        N.check(s._lib.pfg_newmark_setup(s.handle, C.byref(p)))
        n = self.U.shape[0]
        N.check(s._lib.pfg_newmark_set_state(s.handle, n, self.U.ctypes.data, self.V.ctypes.data,
                                             self.A.ctypes.data))
        self._s = s
        self._key = (self.dt, self.Newmark_beta, self.Newmark_gamma, self.alpha, self.beta)

    def LinearReyleighNewmark(self, TOL: float = 1e-10, precision: str = "fp64", storage: str = "full"):
        """One time step (SeismicAnalysis_%LinearReyleighNewmark): U, V, A advance
        with the external acceleration A_ext; the solve stops at |R - A_eff U|/|R| <= TOL."""
        key = (self.dt, self.Newmark_beta, self.Newmark_gamma, self.alpha, self.beta)
        if self._s is None or self._key != key:
            self._setup()
        s = self._s
        opts = s._opts("CG", precision, "BlockJacobi", "true_relative", storage=storage)
        opts.relative_er = float(TOL)
        # a step's warm-started solve takes a few dozen iterations: short CUDA
        # graph chunks stop soon after convergence (measured on GB300, 60^3:
        # 4.0 ms per step with chunks of 8 against 4.65 ms with 32)
        opts.graph_chunk = 8
        n = self.U.shape[0]
        u, v, a, ae = (buf for buf, _ in self._pins)
        if self.A_ext is not ae:  # rebound by the caller: copy into the page-locked buffer
            np.copyto(ae, np.asarray(self.A_ext, dtype=np.float64).reshape(n))
        info = N.Info()
        N.check(s._lib.pfg_newmark_step(s.handle, C.byref(opts), n, ae.ctypes.data, u.ctypes.data,
                                        v.ctypes.data, a.ctypes.data, C.byref(info)))
        self.U, self.V, self.A = u, v, a
        self.last_info = info.as_dict()
        return self.U

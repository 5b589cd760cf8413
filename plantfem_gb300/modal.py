"""ModalAnalysis: plantFEM's ``ModalAnalysis_`` over the GPU path.

Mirrors ``ModalAnalysisClass.f90``: ``init`` (:21-66) numbers the domains'
elements and nodes consecutively, ``setMaterial`` (:68-94) stores per-element
density, Young's modulus and Poisson ratio (a single value broadcasts),
``setBoundary`` (:96-112) removes every DOF of the listed nodes from the
eigenproblem (fix_eig), and ``solve`` (:115-179) assembles the consistent mass
(kept as "B") and the stiffness (kept as "A") and solves K x = lambda M x --
by default every pair by the dense branch of FEMSolver_%eig, as the reference's
``eig`` call does -- giving ``EigenFrequency = sqrt(|lambda|) / 2 / pi`` and
``EigenMode`` (the B-orthonormal vectors, not rescaled).

Several domains are joined in the reference only through an overset penalty
(``setEbOM``), which is outside this path: ``init`` takes one domain.
"""
from __future__ import annotations

import math

import numpy as np

from .femdomain import FEMDomain
from .femsolver import FEMSolver


class ModalAnalysis:
    def __init__(self):
        self.solver: FEMSolver | None = None
        self.domain: FEMDomain | None = None
        self.YoungModulus = self.PoissonRatio = self.Density = None
        self.EigenFrequency = None
        self.EigenMode = None
        self.use_LOBPCG = False  # FEMSolver_%use_LOBPCG of the solver the reference builds
        self.num_eigen: int | None = None
        self.eig_kw: dict = {}
        self._fixed: list[np.ndarray] = []

    def init(self, domains) -> "ModalAnalysis":
        """ModalAnalysis_%init(domains) (ModalAnalysisClass.f90:21-66)."""
        if isinstance(domains, FEMDomain):
            domains = [domains]
        if len(domains) != 1:
            raise NotImplementedError("ModalAnalysis joins several domains only through the overset penalty "
                                      "(setEbOM), which this library does not build: pass one domain")
        self.domain = domains[0]
        ne = self.domain.ne()
        self.YoungModulus = np.zeros(ne)
        self.PoissonRatio = np.zeros(ne)
        self.Density = np.zeros(ne)
        self.solver = FEMSolver()
        self.solver.setDomain(self.domain)
        self.solver.setCRS(3)
        self._fixed = []
        return self

    def setMaterial(self, DomainID: int = 1, Density=None, YoungModulus=None, PoissonRatio=None):
        """ModalAnalysis_%setMaterial (ModalAnalysisClass.f90:68-94): size-1 arrays broadcast."""
        self._check_domain(DomainID)
        for name, v in (("Density", Density), ("YoungModulus", YoungModulus), ("PoissonRatio", PoissonRatio)):
            if v is None:
                continue
            a = np.atleast_1d(np.asarray(v, dtype=np.float64))
            getattr(self, name)[:] = a[0] if a.shape[0] == 1 else a

    def setBoundary(self, DomainID: int = 1, NodeList=None):
        """ModalAnalysis_%setBoundary (ModalAnalysisClass.f90:96-112): the x, y
        and z DOFs of the listed nodes (1-based) leave the eigenproblem."""
        self._check_domain(DomainID)
        nodes = np.asarray(NodeList, dtype=np.int64)
        for d in (1, 2, 3):
            self._fixed.append((nodes - 1) * 3 + d)

    def solve(self, only_matrix: bool = False):
        """ModalAnalysis_%solve (ModalAnalysisClass.f90:115-179)."""
        s = self.solver
        s.zeros()
        s.assembleMass(self.Density)
        s.keepThisMatrixAs("B")
        s.zeros()
        s.assembleStiffness(self.YoungModulus, self.PoissonRatio)
        s.keepThisMatrixAs("A")
        if only_matrix:
            return None
        for ids in self._fixed:
            s.fix_eig(ids)
        s.use_LOBPCG = self.use_LOBPCG
        lam, X = s.eig(self.num_eigen, **self.eig_kw)
        self.EigenFrequency = np.sqrt(np.abs(lam)) / 2.0 / math.pi
        self.EigenMode = X
        return self.EigenFrequency

    def remove(self):
        if self.solver is not None:
            self.solver.remove()
        self.solver = None

    destroy = remove

    @staticmethod
    def _check_domain(DomainID):
        if DomainID != 1:
            raise NotImplementedError("one domain (DomainID = 1)")

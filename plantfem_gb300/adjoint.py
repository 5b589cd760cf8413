"""Differentiable solve: u(E) with dL/dE by one adjoint solve.

The reference has no adjoint; this is the path's differentiation form (dL/dE of
the linear-elastic solve for per-element Young's moduli).
For the eliminated system K(E) u = f (Dirichlet rows/columns removed, as
FEMSolver_%solve does, FEMSolverClass.f90:1707-1756) and a loss L(u),

    dL/dE_e = -lambda^T (dK/dE_e) u,   K lambda = dL/du,  lambda = 0 at fixed DOFs,

and dK/dE_e is the element stiffness at E = 1 (StiffnessMatrixFEMDomain is
linear in E).  The backward pass is one adjoint solve with the same symmetric
matrix plus the element kernel `k_adjoint_grad`; with ``recompute_u`` the
forward solution is recomputed in backward instead of being kept.
"""
from __future__ import annotations

import numpy as np
import torch

from .femsolver import FEMSolver


class ElasticOperator:
    """Mesh, Poisson ratios, load and fixed DOFs of one elasticity problem."""

    def __init__(self, domain, nu, rhs, fix_ids, precision: str = "fp64", relative_er: float = 1e-12,
                 recompute_u: bool = False, algorithm: str = "CG", preconditioning: str = "BlockJacobi",
                 storage: str = "symmetric"):
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.s = FEMSolver()
        self.s.setDomain(domain)
        self.s.setCRS(3)
        self.ne = domain.ne()
        self.n = 3 * domain.nn()
        self.nu = torch.as_tensor(np.broadcast_to(nu, (self.ne,)).copy(), dtype=torch.float64, device=self.dev)
        self.rhs = torch.as_tensor(rhs, dtype=torch.float64, device=self.dev)
        self.fix_ids = np.asarray(fix_ids, dtype=np.int32)
        self.fixed = torch.zeros(self.n, dtype=torch.bool, device=self.dev)
        self.fixed[torch.as_tensor(self.fix_ids.astype(np.int64) - 1, device=self.dev)] = True
        self.s.fix(1, self.fix_ids, FixValue=0.0)
        self.s.relative_er = relative_er
        self.precision = precision
        self.recompute_u = recompute_u
        self.algorithm = algorithm
        self.preconditioning = preconditioning
        # K(E) is symmetric: the mixed inner iterations read its upper half
        self.storage = storage
        self._token = 0      # increases at every assembly
        self._held = None    # token of the matrix the handle holds

    def _assemble(self, E: torch.Tensor) -> int:
        self.s.zeros()
        self.s.assembleStiffness_device(E.contiguous(), self.nu)
        self.s.setRHS_device(self.rhs)
        self.s.eliminate()
        self._token += 1
        self._held = self._token
        return self._token

    def _solve(self, b: torch.Tensor) -> torch.Tensor:
        x = torch.zeros(self.n, dtype=torch.float64, device=self.dev)
        self.s.solve_device(b, x, algorithm=self.algorithm, preconditioning=self.preconditioning,
                            precision=self.precision, stop_rule="true_relative", storage=self.storage)
        self.last_info = self.s.last_info
        return x

    def forward_u(self, E: torch.Tensor) -> torch.Tensor:
        self.last_token = self._assemble(E)
        b = self.rhs.clone()
        b[self.fixed] = 0.0  # eliminated RHS: the fixed values are zero here, so the
        # free rows keep f (f - K_fc u_c with u_c = 0)
        return self._solve(b)

    def displacement(self, E: torch.Tensor) -> torch.Tensor:
        """u(E), differentiable with respect to E (float64 CUDA tensor, one value per element)."""
        return _ElasticSolve.apply(E, self)


class _ElasticSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, E, op: ElasticOperator):
        u = op.forward_u(E)
        ctx.op = op
        ctx.token = op.last_token
        if op.recompute_u:
            ctx.save_for_backward(E)
        else:
            ctx.save_for_backward(E, u)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        op = ctx.op
        saved = ctx.saved_tensors
        E = saved[0]
        if op.recompute_u:
            u = op.forward_u(E)
        else:
            u = saved[1]
            if op._held != ctx.token:  # other forwards re-assembled the handle since
                op._assemble(E)
        b = grad_u.detach().to(torch.float64).contiguous().clone()
        b[op.fixed] = 0.0
        lam = op._solve(b)
        grad = torch.empty(op.ne, dtype=torch.float64, device=op.dev)
        op.s.adjoint_grad_E_device(u.contiguous(), lam, op.nu, grad)
        return grad, None

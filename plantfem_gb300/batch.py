"""FEMSolverBatch: many FEMSolver systems solved in one persistent launch.

plantFEM solves one organ mesh per ``FEMSolver_`` object and calls
``FEMSolver_%solve`` on each in turn (FEMSolverClass.f90:1697-1825).  Here the
same objects, set up exactly as for ``solve`` (setDomain, setCRS, assembly,
fix), are bound to a batch and solved together by one persistent CUDA kernel
(``pfg_batch_*`` in include/pfg.h): one CTA per system, or a thread-block
cluster for the largest ones, with jobs taken largest-first from an atomic
queue.  The launch configuration is picked by :meth:`tune`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .femsolver import FEMSolver

_PC = {None: N.PC_NONE, "None": N.PC_NONE, "PointJacobi": N.PC_JACOBI, "Jacobi": N.PC_JACOBI,
       "BlockJacobi": N.PC_BLOCK_JACOBI}
_PREC = {"fp64": N.PREC_FP64, "FP64": N.PREC_FP64, "mixed": N.PREC_MIXED}


class FEMSolverBatch:
    def __init__(self, solvers=None):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.pfg_batch_create(C.byref(h)))
        self._h = h
        self.solvers: list[FEMSolver] = []
        self._ndof: list[int] = []
        self.last_infos: list[dict] = []
        self.last_info: dict = {}
        if solvers is not None:
            self.set(solvers)

    def __del__(self):
        try:
            if self._h:
                self._lib.pfg_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def set(self, solvers) -> "FEMSolverBatch":
        """Bind the systems (eliminates each one as FEMSolver_%solve does)."""
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.handle.value for s in self.solvers])
        N.check(self._lib.pfg_batch_set(self._h, len(self.solvers), arr))
        self._ndof = [s.ndof() for s in self.solvers]
        return self

    def _opts(self, precision, preconditioning, relative_er, itrmax, reliable_delta, debug=False):
        o = N.default_opts(algorithm=N.ALG_CG, precision=_PREC[precision], precond=_PC[preconditioning],
                           stop_rule=N.STOP_TRUE_RELATIVE, relative_er=float(relative_er), itrmax=int(itrmax),
                           debug=int(bool(debug)))
        if reliable_delta is not None:
            o.reliable_delta = float(reliable_delta)
        return o

    def solve(self, precision: str = "mixed", preconditioning: str | None = "BlockJacobi",
              relative_er: float = 1e-10, itrmax: int = 100000, reliable_delta: float | None = None,
              return_x: bool = True):
        """Solve every bound system; returns the list of displacement vectors
        (or None with ``return_x=False``: the solutions stay on the device,
        :meth:`get_x` reads one).  Per-system records in ``last_infos``."""
        o = self._opts(precision, preconditioning, relative_er, itrmax, reliable_delta)
        n = len(self.solvers)
        infos = (N.Info * n)()
        bi = N.BatchInfo()
        xs = None
        xp = None
        if return_x:
            xs = [np.zeros(k) for k in self._ndof]
            xp = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        N.check(self._lib.pfg_batch_solve(self._h, C.byref(o), xp, infos, C.byref(bi)))
        self.last_infos = [i.as_dict() for i in infos]
        self.last_info = bi.as_dict()
        return xs

    def get_x(self, index: int) -> np.ndarray:
        x = np.zeros(self._ndof[index])
        N.check(self._lib.pfg_batch_get_x(self._h, int(index), x.ctypes.data))
        return x

    @property
    def config(self) -> dict:
        c = N.BatchConfig()
        t = C.c_int32()
        N.check(self._lib.pfg_batch_get_config(self._h, C.byref(c), C.byref(t)))
        d = c.as_dict()
        d["tuned"] = bool(t.value)
        return d

    @config.setter
    def config(self, cfg: dict):
        c = N.BatchConfig(int(cfg["threads"]), int(cfg["cluster"]), float(cfg["team_fraction"]))
        N.check(self._lib.pfg_batch_set_config(self._h, C.byref(c)))

    def tune(self, precision: str = "mixed", preconditioning: str | None = "BlockJacobi",
             relative_er: float = 1e-10, itrmax: int = 100000, debug: bool = False) -> tuple[dict, float]:
        """Autotune the launch configuration on the bound systems; returns (config, ms).
        ``debug`` prints every candidate's time on stderr."""
        o = self._opts(precision, preconditioning, relative_er, itrmax, None, debug)
        c = N.BatchConfig()
        ms = C.c_double()
        N.check(self._lib.pfg_batch_tune(self._h, C.byref(o), C.byref(c), C.byref(ms)))
        return c.as_dict(), ms.value

    def abort_flag(self):
        """ctypes pointer to the host-mapped abort flag (set [0] = 1 to abort)."""
        p = C.POINTER(C.c_int32)()
        N.check(self._lib.pfg_batch_abort_flag(self._h, C.byref(p)))
        return p

"""GB300 (sm_103a) PDHG LP engine.

Drop-in for the GPU PDHG path of the reference's ``sih_solver`` package
(py/sih_solver/__init__.py:81-91): ``GpuSolver.solve_pdhg``,
``GpuSolver.is_cuda_available``, ``GpuSolver.get_vram_info``,
``solve_gpu_pdhg`` and ``GpuPdhgConfig`` keep their names and meaning, over the
C ABI of include/sih_pdhg.h.  Added: ``GpuSolver.solve_ex`` / ``solve_gpu_mixed``
(mixed-precision restarted adaptive PDHG).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ALGO_MIXED, ALGO_PLAIN, SihPdhgError, default_options
from .config import GpuPdhgConfig
from .problem import INF, ObjectiveSense, Problem, Solution, SolutionStatus, SparseMatrix

__all__ = ["GpuSolver", "GpuPdhgConfig", "GpuMemoryInfo", "Problem", "SparseMatrix", "Solution",
           "SolutionStatus", "ObjectiveSense", "solve_gpu_pdhg", "solve_gpu_mixed", "default_options",
           "SihPdhgError", "ALGO_PLAIN", "ALGO_MIXED", "INF"]


@dataclass
class GpuMemoryInfo:
    """Fields of ``sih::gpu::GpuMemoryInfo`` (gpu_solver.hpp:24-28)."""
    total_bytes: int = 0
    free_bytes: int = 0
    used_bytes: int = 0


def _solve(problem: Problem, config: GpuPdhgConfig, opts) -> Solution:
    lib = _lib.load()
    m, n = problem.num_rows(), problem.num_cols()
    x = np.zeros(n)
    y = np.zeros(m)
    slack = np.zeros(m)
    rc = np.zeros(n)
    cp, keep = _lib.c_problem(problem)
    res = _lib.CResult()
    res.x, res.row_duals, res.slack, res.reduced_costs = x.ctypes.data, y.ctypes.data, slack.ctypes.data, rc.ctypes.data
    if opts is None:
        _lib.check(lib.sih_pdhg_solve(C.byref(cp), C.byref(config), C.byref(res)))
    else:
        _lib.check(lib.sih_pdhg_solve_ex(C.byref(cp), C.byref(config), C.byref(opts), C.byref(res)))
    del keep
    return Solution(status=SolutionStatus(res.status), x=x, slack=slack, row_duals=y, reduced_costs=rc,
                    primal_objective=res.primal_objective, dual_bound=res.dual_bound,
                    simplex_iterations=int(res.iterations), time_wall_sec=res.time_wall_sec,
                    time_solver_sec=res.time_solver_sec, rel_primal=res.rel_primal, rel_dual=res.rel_dual,
                    rel_gap=res.rel_gap, ref_primal=res.ref_primal, ref_dual=res.ref_dual,
                    restarts=int(res.restarts), step_rejections=int(res.step_rejections),
                    final_step=res.final_step, final_primal_weight=res.final_primal_weight)


class GpuSolver:
    """Static entry points of ``sih::gpu::GpuSolver`` (gpu_solver.hpp:30-45)."""

    @staticmethod
    def is_cuda_available() -> bool:
        return bool(_lib.load().sih_pdhg_is_cuda_available())

    @staticmethod
    def get_vram_info() -> GpuMemoryInfo:
        if not GpuSolver.is_cuda_available():
            return GpuMemoryInfo()
        t, f, u = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _lib.check(_lib.load().sih_pdhg_get_vram_info(C.byref(t), C.byref(f), C.byref(u)))
        return GpuMemoryInfo(t.value, f.value, u.value)

    @staticmethod
    def solve_pdhg(problem: Problem, config: Optional[GpuPdhgConfig] = None) -> Solution:
        """The reference's FP32 PDHG (gpu_solver.cpp:60-307) on the GPU."""
        return _solve(problem, config if config is not None else GpuPdhgConfig(), None)

    @staticmethod
    def solve_ex(problem: Problem, config: Optional[GpuPdhgConfig] = None, **options) -> Solution:
        """Solve with the added options (``algorithm=ALGO_MIXED`` etc., see sih_pdhg_options)."""
        return _solve(problem, config if config is not None else GpuPdhgConfig(), default_options(**options))


def solve_gpu_pdhg(problem: Problem, config: Optional[GpuPdhgConfig] = None) -> Solution:
    """Solve an LP with the GPU PDHG engine (py/sih_solver/__init__.py:81-85)."""
    return GpuSolver.solve_pdhg(problem, config)


def solve_gpu_mixed(problem: Problem, config: Optional[GpuPdhgConfig] = None, **options) -> Solution:
    """Mixed-precision restarted adaptive PDHG (rel. KKT termination at tol_primal/tol_dual/tol_gap)."""
    options.setdefault("algorithm", ALGO_MIXED)
    return GpuSolver.solve_ex(problem, config, **options)

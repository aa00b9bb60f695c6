"""GB300 (sm_103a) PDHG LP engine.

Drop-in for the GPU PDHG path of the reference's ``sih_solver`` package
(py/sih_solver/__init__.py:81-91): ``GpuSolver.solve_pdhg``,
``GpuSolver.is_cuda_available``, ``GpuSolver.get_vram_info``,
``solve_gpu_pdhg`` and ``GpuPdhgConfig`` keep their names and meaning, over the
C ABI of include/sih_pdhg.h.  Added: ``GpuSolver.solve_ex`` / ``solve_gpu_mixed``
(mixed-precision restarted adaptive PDHG), ``read_mps`` (the reference's
``sih_solver.read_mps`` records, core/src/io/mps_io.cpp:63-323, read by the
engine's one-pass MPS reader).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ALGO_MIXED, ALGO_PLAIN, SihPdhgError, default_options
from .config import GpuPdhgConfig
from .mps import write_mps
from .problem import INF, ObjectiveSense, Problem, Solution, SolutionStatus, SparseMatrix

__all__ = ["GpuSolver", "GpuPdhgConfig", "GpuMemoryInfo", "Problem", "SparseMatrix", "Solution",
           "SolutionStatus", "ObjectiveSense", "solve_gpu_pdhg", "solve_gpu_mixed", "solve_batch", "PdhgHandle",
           "default_options", "SihPdhgError", "ALGO_PLAIN", "ALGO_MIXED", "INF", "adjoint_batch", "polish_batch",
           "read_mps", "read_mps_text", "write_mps"]


@dataclass
class GpuMemoryInfo:
    """Fields of ``sih::gpu::GpuMemoryInfo`` (gpu_solver.hpp:24-28)."""
    total_bytes: int = 0
    free_bytes: int = 0
    used_bytes: int = 0


def _result_buffers(problem: Problem):
    m, n = problem.num_rows(), problem.num_cols()
    bufs = dict(x=np.zeros(n), row_duals=np.zeros(m), slack=np.zeros(m), reduced_costs=np.zeros(n))
    res = _lib.CResult()
    res.x, res.row_duals = bufs["x"].ctypes.data, bufs["row_duals"].ctypes.data
    res.slack, res.reduced_costs = bufs["slack"].ctypes.data, bufs["reduced_costs"].ctypes.data
    return res, bufs


def _to_solution(res, bufs) -> Solution:
    sol = Solution(status=SolutionStatus(res.status), primal_objective=res.primal_objective,
                   dual_bound=res.dual_bound, simplex_iterations=int(res.iterations),
                   time_wall_sec=res.time_wall_sec, time_solver_sec=res.time_solver_sec,
                   rel_primal=res.rel_primal, rel_dual=res.rel_dual, rel_gap=res.rel_gap,
                   ref_primal=res.ref_primal, ref_dual=res.ref_dual, restarts=int(res.restarts),
                   step_rejections=int(res.step_rejections), final_step=res.final_step,
                   final_primal_weight=res.final_primal_weight, **bufs)
    sol.h2d_bytes = int(res.h2d_bytes)
    sol.d2h_bytes = int(res.d2h_bytes)
    sol.kernel_launches = int(res.kernel_launches)
    return sol


def _solve(problem: Problem, config: GpuPdhgConfig, opts) -> Solution:
    lib = _lib.load()
    cp, keep = _lib.c_problem(problem)
    res, bufs = _result_buffers(problem)
    if opts is None:
        _lib.check(lib.sih_pdhg_solve(C.byref(cp), C.byref(config), C.byref(res)))
    else:
        _lib.check(lib.sih_pdhg_solve_ex(C.byref(cp), C.byref(config), C.byref(opts), C.byref(res)))
    del keep
    return _to_solution(res, bufs)


class PdhgHandle:
    """One LP or a batch of LPs kept resident on the GPU (sih_pdhg_create / run /
    get_result / destroy).  The problems must outlive the handle."""

    def __init__(self, problems, config: Optional[GpuPdhgConfig] = None, **options):
        self._lib = _lib.load()
        self.problems = list(problems) if isinstance(problems, (list, tuple)) else [problems]
        self.config = config if config is not None else GpuPdhgConfig()
        self.options = default_options(**options)
        views = [_lib.c_problem(p) for p in self.problems]
        self._keep = [v[1] for v in views]
        arr = (_lib.CProblem * len(views))(*[v[0] for v in views])
        self._arr = arr
        h = C.c_void_p()
        _lib.check(self._lib.sih_pdhg_create(arr, len(views), C.byref(self.config), C.byref(self.options),
                                             C.byref(h)))
        self._h = h

    def run(self) -> float:
        """Solves every instance from its initial point; returns the device seconds."""
        secs = C.c_double()
        _lib.check(self._lib.sih_pdhg_run(self._h, C.byref(secs)))
        return secs.value

    def result(self, index: int = 0) -> Solution:
        if not 0 <= index < len(self.problems):
            raise SihPdhgError(1, f"index {index} out of range")
        res, bufs = _result_buffers(self.problems[index])
        _lib.check(self._lib.sih_pdhg_get_result(self._h, index, C.byref(res)))
        return _to_solution(res, bufs)

    def time_kernels(self, reps: int = 10):
        """Average seconds and algorithmic bytes per launch of the three step kernels
        (elementwise primal step, A x rows step, A^T y columns step)."""
        secs = (C.c_double * 3)()
        byts = (C.c_double * 3)()
        _lib.check(self._lib.sih_pdhg_time_kernels(self._h, reps, secs, byts))
        return list(secs), list(byts)

    def set_start(self, index: int, x, row_duals=None, primal_weight: float = 0.0) -> None:
        """Warm start of instance `index` for the following runs (x in the
        original column order, row_duals in the returned convention; None
        clears it).  Pass a previous Solution's x, row_duals and
        final_primal_weight to re-solve a perturbed scenario."""
        if x is None:
            _lib.check(self._lib.sih_pdhg_set_start(self._h, index, None, None, 0.0))
            return
        xa = np.ascontiguousarray(x, dtype=np.float64)
        ya = None if row_duals is None else np.ascontiguousarray(row_duals, dtype=np.float64)
        p = self.problems[index] if 0 <= index < len(self.problems) else None
        if p is not None and (xa.shape != (p.num_cols(),) or (ya is not None and ya.shape != (p.num_rows(),))):
            raise SihPdhgError(1, "start vectors do not match the instance's shape")
        _lib.check(self._lib.sih_pdhg_set_start(self._h, index, xa.ctypes.data,
                                                None if ya is None else ya.ctypes.data, float(primal_weight)))

    def task_nnz(self) -> int:
        """Nonzeros per SpMV task in use (the autotuner's choice with autotune=1)."""
        v = C.c_int32()
        _lib.check(self._lib.sih_pdhg_get_task_nnz(self._h, C.byref(v)))
        return v.value

    def launch_shape(self) -> dict:
        """Launch shape of the step kernels (sih_pdhg_get_launch_shape): task size,
        lanes per segment of each side, staged gathers, step form, grid, and
        whether the autotuner chose it."""
        sh = _lib.CLaunchShape()
        _lib.check(self._lib.sih_pdhg_get_launch_shape(self._h, C.byref(sh)))
        return {f: getattr(sh, f) for f, _ in _lib.CLaunchShape._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sih_pdhg_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()


def solve_batch(problems, config: Optional[GpuPdhgConfig] = None, **options):
    """Solves a list of LPs in one batched launch sequence (sih_pdhg_solve_batch)."""
    lib = _lib.load()
    options.setdefault("algorithm", ALGO_MIXED)
    opts = default_options(**options)
    config = config if config is not None else GpuPdhgConfig()
    views = [_lib.c_problem(p) for p in problems]
    arr = (_lib.CProblem * len(views))(*[v[0] for v in views])
    outs = [_result_buffers(p) for p in problems]
    res_arr = (_lib.CResult * len(problems))(*[o[0] for o in outs])
    _lib.check(lib.sih_pdhg_solve_batch(arr, len(views), C.byref(config), C.byref(opts), res_arr))
    return [_to_solution(res_arr[i], outs[i][1]) for i in range(len(problems))]


def adjoint_batch(problems, xs, row_duals, grad_xs, tolerance: float = 1e-6, max_iterations: int = 0):
    """Gradients of a loss with respect to the LP data, from the loss gradient
    with respect to each solution x (sih_pdhg_adjoint_batch).  `row_duals` as
    returned with the default dual_sign.  Returns (grads, infos): grads[i] is a
    dict with c, row_lower, row_upper, col_lower, col_upper (float64 arrays)."""
    lib = _lib.load()
    problems = list(problems)
    B = len(problems)
    views = [_lib.c_problem(p) for p in problems]
    arr = (_lib.CProblem * B)(*[v[0] for v in views])
    keep = [v[1] for v in views]
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    xs = [f64(a) for a in xs]
    ys = [f64(a) for a in row_duals]
    gs = [f64(a) for a in grad_xs]
    for p, x, y, g in zip(problems, xs, ys, gs):
        if x.shape != (p.num_cols(),) or g.shape != (p.num_cols(),) or y.shape != (p.num_rows(),):
            raise SihPdhgError(1, "x / grad_x need num_cols entries and row_duals num_rows")
    out = [{k: np.zeros(p.num_cols() if k in ("c", "col_lower", "col_upper") else p.num_rows())
            for k in ("c", "row_lower", "row_upper", "col_lower", "col_upper")} for p in problems]
    ptrs = lambda lst: (C.c_void_p * B)(*[a.ctypes.data for a in lst])
    opts = _lib.CAdjointOptions()
    lib.sih_pdhg_adjoint_options_default(C.byref(opts))
    opts.tolerance = float(tolerance)
    opts.max_iterations = int(max_iterations)
    infos = (_lib.CAdjointInfo * B)()
    _lib.check(lib.sih_pdhg_adjoint_batch(
        arr, B, ptrs(xs), ptrs(ys), ptrs(gs), ptrs([o["c"] for o in out]), ptrs([o["row_lower"] for o in out]),
        ptrs([o["row_upper"] for o in out]), ptrs([o["col_lower"] for o in out]), ptrs([o["col_upper"] for o in out]),
        C.byref(opts), infos))
    del keep
    return out, [{k: getattr(infos[i], k) for k, _ in _lib.CAdjointInfo._fields_ if k != "reserved"}
                 for i in range(B)]


def basis_guess(problem: Problem, x, row_activity):
    """Basis guess of the hybrid polish on the GPU (sih_pdhg_basis_guess; the
    scoring of GpuSolver::solve_hybrid, core/src/gpu/gpu_solver.cpp:332-395):
    the m columns / rows farthest from their nearer finite bound are Basic (0),
    the others AtLower (1) or AtUpper (2).  Returns (col_status, row_status) as
    int8 arrays, values of sih::model::BasisStatus."""
    lib = _lib.load()
    cp, keep = _lib.c_problem(problem)
    xa = np.ascontiguousarray(x, dtype=np.float64)
    ax = np.ascontiguousarray(row_activity, dtype=np.float64)
    if xa.shape != (problem.num_cols(),) or ax.shape != (problem.num_rows(),):
        raise SihPdhgError(1, "x / row_activity do not match the problem's shape")
    cs = np.empty(problem.num_cols(), dtype=np.int8)
    rs = np.empty(problem.num_rows(), dtype=np.int8)
    _lib.check(lib.sih_pdhg_basis_guess(C.byref(cp), xa.ctypes.data, ax.ctypes.data, cs.ctypes.data, rs.ctypes.data))
    return cs, rs


def polish_batch(problems, xs, row_duals, tolerance: float = 1e-6, max_iterations: int = 0):
    """Basis polish (sih_pdhg_polish_batch): the vertex and duals of the basis
    read off each PDHG point.  Returns (xs_out, duals_out, infos)."""
    lib = _lib.load()
    problems = list(problems)
    B = len(problems)
    views = [_lib.c_problem(p) for p in problems]
    arr = (_lib.CProblem * B)(*[v[0] for v in views])
    keep = [v[1] for v in views]
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    xs = [f64(a) for a in xs]
    ys = [f64(a) for a in row_duals]
    for p, x, y in zip(problems, xs, ys):
        if x.shape != (p.num_cols(),) or y.shape != (p.num_rows(),):
            raise SihPdhgError(1, "x needs num_cols entries and row_duals num_rows")
    xo = [np.zeros(p.num_cols()) for p in problems]
    yo = [np.zeros(p.num_rows()) for p in problems]
    ptrs = lambda lst: (C.c_void_p * B)(*[a.ctypes.data for a in lst])
    opts = _lib.CAdjointOptions()
    lib.sih_pdhg_adjoint_options_default(C.byref(opts))
    opts.tolerance = float(tolerance)
    opts.max_iterations = int(max_iterations)
    infos = (_lib.CPolishInfo * B)()
    _lib.check(lib.sih_pdhg_polish_batch(arr, B, ptrs(xs), ptrs(ys), ptrs(xo), ptrs(yo), C.byref(opts), infos))
    del keep
    return xo, yo, [{k: getattr(infos[i], k) for k, _ in _lib.CPolishInfo._fields_ if k != "reserved"}
                    for i in range(B)]



def _problem_from_mps(handle) -> Problem:
    lib = _lib.load()
    view = _lib.CProblem()
    name = C.c_char_p()
    ints = C.c_int64()
    try:
        _lib.check(lib.sih_pdhg_mps_view(handle, C.byref(view), C.byref(name), C.byref(ints)))
        m, n, nnz = view.num_rows, view.num_cols, view.num_nonzeros

        def arr(ptr, count, ctype):
            if count == 0:
                return np.zeros(0, dtype=np.int64 if ctype is C.c_int64 else np.float64)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()

        A = SparseMatrix(m, n, arr(view.csc_col_ptr, n + 1, C.c_int64), arr(view.csc_row_ind, nnz, C.c_int64),
                         arr(view.csc_values, nnz, C.c_double), arr(view.csr_row_ptr, m + 1, C.c_int64),
                         arr(view.csr_col_ind, nnz, C.c_int64), arr(view.csr_values, nnz, C.c_double))
        p = Problem.from_arrays(A, arr(view.c, n, C.c_double), arr(view.col_lower, n, C.c_double),
                                arr(view.col_upper, n, C.c_double), arr(view.row_lower, m, C.c_double),
                                arr(view.row_upper, m, C.c_double), ObjectiveSense(view.sense), view.obj_offset,
                                (name.value or b"").decode(errors="replace"))
        p.integer_columns = int(ints.value)
        return p
    finally:
        lib.sih_pdhg_mps_free(handle)


def read_mps(path) -> Problem:
    """Problem of an MPS file (sih_pdhg_read_mps): the records of the reference's
    reader, CSC and CSR filled.  ``problem.integer_columns`` counts integer
    columns (solved as their LP relaxation).  Raises SihPdhgError on a parse
    error or a quadratic objective."""
    lib = _lib.load()
    h = C.c_void_p()
    _lib.check(lib.sih_pdhg_read_mps(str(path).encode(), C.byref(h)))
    return _problem_from_mps(h)


def read_mps_text(text) -> Problem:
    """read_mps of an MPS text held in memory (str or bytes)."""
    lib = _lib.load()
    data = text.encode() if isinstance(text, str) else bytes(text)
    h = C.c_void_p()
    _lib.check(lib.sih_pdhg_read_mps_text(data, len(data), C.byref(h)))
    return _problem_from_mps(h)


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

"""LP problem and solution containers for the GB300 PDHG engine.

These mirror the parts of the reference model layer that the GPU PDHG path
reads and writes:

* ``Problem`` follows ``sih::model::Problem`` (core/include/sih/model/problem.hpp:37-137):
  dimensions, objective ``c`` with ``sense``/``obj_offset``, row bounds
  ``row_lower``/``row_upper`` and column bounds ``col_lower``/``col_upper``.
* ``SparseMatrix`` follows ``sih::model::SparseMatrix``
  (core/include/sih/model/sparse_matrix.hpp:20-77): the matrix is held twice,
  as CSC and as CSR, with int64 indices and float64 values, rows ascending
  within a column and columns ascending within a row (the order produced by
  ``SparseMatrix::from_triplets``, core/src/model/sparse_matrix.cpp:43-85).
* ``Solution`` carries the fields ``GpuSolver::solve_pdhg`` fills
  (core/src/gpu/gpu_solver.cpp:290-304) plus the ones the reference leaves
  empty (slack, reduced costs, dual bound) and the relative KKT triple.

Infinite bounds are IEEE infinities, as in the reference (``SIH_INFINITY``).
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

INF = float("inf")


class ObjectiveSense(enum.IntEnum):
    """Same values as ``sih::model::ObjectiveSense`` (problem.hpp:14-17)."""
    Minimize = 1
    Maximize = -1


class SolutionStatus(enum.IntEnum):
    """Same values as ``sih::model::SolutionStatus`` (solution.hpp:11-21)."""
    Optimal = 0
    Infeasible = 1
    Unbounded = 2
    TimeLimit = 3
    IterationLimit = 4
    NodeLimit = 5
    NumericalFailure = 6
    Interrupted = 7
    Unknown = 8


class SparseMatrix:
    """Dual CSC + CSR storage with int64 indices and float64 values."""

    def __init__(self, rows: int, cols: int, csc_col_ptr, csc_row_ind, csc_values,
                 csr_row_ptr=None, csr_col_ind=None, csr_values=None):
        self._m = int(rows)
        self._n = int(cols)
        self._cp = np.ascontiguousarray(csc_col_ptr, dtype=np.int64)
        self._ri = np.ascontiguousarray(csc_row_ind, dtype=np.int64)
        self._cv = np.ascontiguousarray(csc_values, dtype=np.float64)
        if self._cp.shape != (self._n + 1,):
            raise ValueError("csc_col_ptr must have num_cols + 1 entries")
        if self._ri.shape != self._cv.shape or self._ri.shape[0] != int(self._cp[-1]):
            raise ValueError("csc_row_ind / csc_values length must equal csc_col_ptr[-1]")
        self._rp = self._ci = self._rv = None
        if csr_row_ptr is not None:
            self._set_csr(csr_row_ptr, csr_col_ind, csr_values)

    def _set_csr(self, rp, ci, rv) -> None:
        self._rp = np.ascontiguousarray(rp, dtype=np.int64)
        self._ci = np.ascontiguousarray(ci, dtype=np.int64)
        self._rv = np.ascontiguousarray(rv, dtype=np.float64)
        if self._rp.shape != (self._m + 1,) or self._ci.shape[0] != self._ri.shape[0]:
            raise ValueError("CSR arrays do not match the CSC arrays")

    def has_csr(self) -> bool:
        """True once the CSR copy exists (it is built on first use; the engine
        builds its own when a problem arrives without one)."""
        return self._rp is not None

    def _csr(self):
        if self._rp is None:
            self._set_csr(*csc_to_csr(self._m, self._n, self._cp, self._ri, self._cv))
        return self._rp, self._ci, self._rv

    @staticmethod
    def from_triplets(m: int, n: int, rows, cols, vals, zero_tol: float = 1e-15) -> "SparseMatrix":
        """Sum duplicates, drop |v| <= zero_tol, build CSC and CSR
        (as ``SparseMatrix::from_triplets``, sparse_matrix.cpp:13-88)."""
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        vals = np.asarray(vals, dtype=np.float64)
        if rows.size and (rows.min() < 0 or rows.max() >= m or cols.min() < 0 or cols.max() >= n):
            raise IndexError("Triplet indices out of matrix bounds")
        key = cols * max(m, 1) + rows
        uniq, inv = np.unique(key, return_inverse=True)
        summed = np.zeros(uniq.shape[0], dtype=np.float64)
        np.add.at(summed, inv, vals)
        keep = np.abs(summed) > zero_tol
        uniq, summed = uniq[keep], summed[keep]
        c = uniq // max(m, 1)
        r = uniq % max(m, 1)
        cp = np.zeros(n + 1, dtype=np.int64)
        np.add.at(cp, c + 1, 1)
        np.cumsum(cp, out=cp)
        return SparseMatrix(m, n, cp, r, summed)

    def num_rows(self) -> int:
        return self._m

    def num_cols(self) -> int:
        return self._n

    def num_nonzeros(self) -> int:
        return int(self._ri.shape[0])

    def csc_col_ptr(self):
        return self._cp

    def csc_row_ind(self):
        return self._ri

    def csc_values(self):
        return self._cv

    def csr_row_ptr(self):
        return self._csr()[0]

    def csr_col_ind(self):
        return self._csr()[1]

    def csr_values(self):
        return self._csr()[2]

    def mat_vec(self, x) -> np.ndarray:
        """y = A x in float64 (as ``SparseMatrix::mat_vec``, sparse_matrix.cpp:90-104)."""
        x = np.asarray(x, dtype=np.float64)
        rp, ci, rv = self._csr()
        rows = np.repeat(np.arange(self._m, dtype=np.int64), np.diff(rp))
        return np.bincount(rows, weights=rv * x[ci], minlength=self._m)

    def mat_trans_vec(self, y) -> np.ndarray:
        """z = A^T y in float64 (as ``SparseMatrix::mat_trans_vec``, sparse_matrix.cpp:115-129)."""
        y = np.asarray(y, dtype=np.float64)
        cols = np.repeat(np.arange(self._n, dtype=np.int64), np.diff(self._cp))
        return np.bincount(cols, weights=self._cv * y[self._ri], minlength=self._n)


def csc_to_csr(m, n, cp, ri, cv):
    """Counting-sort transpose that keeps columns ascending within each row."""
    cp = np.asarray(cp, dtype=np.int64)
    ri = np.asarray(ri, dtype=np.int64)
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(cp))
    order = np.lexsort((cols, ri))
    rp = np.zeros(m + 1, dtype=np.int64)
    np.add.at(rp, ri + 1, 1)
    np.cumsum(rp, out=rp)
    return rp, cols[order], np.asarray(cv, dtype=np.float64)[order]


class Problem:
    """Continuous LP: min/max sense*c^T x + offset, row_lower <= A x <= row_upper,
    col_lower <= x <= col_upper."""

    def __init__(self, name: str = "problem"):
        self.name = name
        self.sense = ObjectiveSense.Minimize
        self.obj_offset = 0.0
        self.c = np.zeros(0)
        self.A = SparseMatrix(0, 0, np.zeros(1, np.int64), np.zeros(0, np.int64), np.zeros(0))
        self.row_lower = np.zeros(0)
        self.row_upper = np.zeros(0)
        self.col_lower = np.zeros(0)
        self.col_upper = np.zeros(0)
        self.integer_columns = 0  # integer columns of an MPS file (solved as their LP relaxation)

    @staticmethod
    def from_arrays(A: SparseMatrix, c, col_lower, col_upper, row_lower, row_upper,
                    sense: ObjectiveSense = ObjectiveSense.Minimize, obj_offset: float = 0.0,
                    name: str = "problem") -> "Problem":
        p = Problem(name)
        p.A = A
        p.c = np.ascontiguousarray(c, dtype=np.float64)
        p.col_lower = np.ascontiguousarray(col_lower, dtype=np.float64)
        p.col_upper = np.ascontiguousarray(col_upper, dtype=np.float64)
        p.row_lower = np.ascontiguousarray(row_lower, dtype=np.float64)
        p.row_upper = np.ascontiguousarray(row_upper, dtype=np.float64)
        p.sense = ObjectiveSense(sense)
        p.obj_offset = float(obj_offset)
        p.validate()
        return p

    def num_rows(self) -> int:
        return self.A.num_rows()

    def num_cols(self) -> int:
        return self.A.num_cols()

    def num_nonzeros(self) -> int:
        return self.A.num_nonzeros()

    def validate(self) -> None:
        m, n = self.num_rows(), self.num_cols()
        for name, arr, ln in (("c", self.c, n), ("col_lower", self.col_lower, n), ("col_upper", self.col_upper, n),
                              ("row_lower", self.row_lower, m), ("row_upper", self.row_upper, m)):
            if arr.shape != (ln,):
                raise ValueError(f"{name} has shape {arr.shape}, expected ({ln},)")


@dataclass
class Solution:
    """Result of a PDHG solve (fields of ``sih::model::Solution``, solution.hpp:37-84)."""
    status: SolutionStatus = SolutionStatus.Unknown
    x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    slack: np.ndarray = field(default_factory=lambda: np.zeros(0))
    row_duals: np.ndarray = field(default_factory=lambda: np.zeros(0))
    reduced_costs: np.ndarray = field(default_factory=lambda: np.zeros(0))
    primal_objective: float = 0.0
    dual_bound: float = 0.0
    simplex_iterations: int = 0
    time_wall_sec: float = 0.0
    time_solver_sec: float = 0.0
    # relative KKT triple of the returned point (docs/gpu_pdhg.md:51-57 definitions, FP64)
    rel_primal: float = float("nan")
    rel_dual: float = float("nan")
    rel_gap: float = float("nan")
    # the reference's own termination measures (gpu_solver.cpp:252-259) at the last check
    ref_primal: float = float("nan")
    ref_dual: float = float("nan")
    restarts: int = 0
    step_rejections: int = 0
    final_step: float = 0.0
    final_primal_weight: float = 0.0

    def is_optimal(self) -> bool:
        return self.status == SolutionStatus.Optimal

    def is_feasible(self) -> bool:
        return self.status in (SolutionStatus.Optimal, SolutionStatus.TimeLimit,
                               SolutionStatus.IterationLimit, SolutionStatus.NodeLimit)

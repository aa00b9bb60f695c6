"""Seeded synthetic LP generators for the PDHG workloads.

All generators are deterministic functions of ``seed`` (numpy ``default_rng``)
and return a :class:`~sih_pdhg.problem.Problem` whose data is float64 with
int64 CSC/CSR indices, like the reference model layer.

``random_feasible_lp`` is the "feasible by construction" recipe:

* column ``j`` holds ``counts[j]`` nonzeros at distinct uniform-random rows,
  values ~ N(0, 1);
* bounds ``0 <= x <= U`` with ``U ~ Uniform(1, 10)``;
* ``x0 ~ Uniform(0, U)``; the first ``m_eq`` rows are equalities ``A x = A x0``,
  the rest are ``A x <= A x0 + Uniform(0, 1)``;
* ``y0 ~ N(0, 1)`` with ``y0 <= 0`` on the ``<=`` rows, ``c = A^T y0 + s``,
  ``s ~ Uniform(0, 1)``.

The draws are made in the fixed order: column counts (Zipf variant only),
row indices (with redraws of duplicates), values, U, x0, slack, y0, s.
"""
from __future__ import annotations

import numpy as np

from .problem import INF, ObjectiveSense, Problem, SparseMatrix, csc_to_csr


def _distinct_rows(rng: np.random.Generator, counts: np.ndarray, m: int):
    """Row indices for each column, distinct within a column, sorted ascending."""
    n = counts.shape[0]
    cols = np.repeat(np.arange(n, dtype=np.int64), counts)
    rows = rng.integers(0, m, size=cols.shape[0], dtype=np.int64)
    while True:
        key = cols * m + rows
        order = np.argsort(key, kind="stable")
        sk = key[order]
        dup = np.zeros(sk.shape[0], dtype=bool)
        dup[1:] = sk[1:] == sk[:-1]
        if not dup.any():
            break
        idx = order[dup]
        rows[idx] = rng.integers(0, m, size=idx.shape[0], dtype=np.int64)
    order = np.lexsort((rows, cols))
    return cols[order], rows[order]


def zipf_column_counts(rng: np.random.Generator, n: int, nnz: int, a: float = 1.5,
                       lo: int = 2, hi: int = 2000) -> np.ndarray:
    """Column counts ~ Zipf(a) clipped to [lo, hi], rescaled (stochastic rounding)
    so that they sum to exactly ``nnz``, re-clipped to [lo, hi]."""
    k = np.clip(rng.zipf(a, n), lo, hi).astype(np.float64)
    k *= nnz / k.sum()
    k = np.clip(np.floor(k + rng.random(n)), lo, hi).astype(np.int64)
    diff = int(nnz - k.sum())
    while diff != 0:
        if diff > 0:
            cand = np.flatnonzero(k < hi)
            pick = rng.choice(cand, size=min(diff, cand.shape[0]), replace=False)
            k[pick] += 1
        else:
            cand = np.flatnonzero(k > lo)
            pick = rng.choice(cand, size=min(-diff, cand.shape[0]), replace=False)
            k[pick] -= 1
        diff = int(nnz - k.sum())
    return k


def random_feasible_lp(m: int, n: int, counts, seed: int = 0, m_eq: int | None = None,
                       name: str = "random_lp", rng: np.random.Generator | None = None) -> Problem:
    rng = np.random.default_rng(seed) if rng is None else rng
    counts = np.asarray(counts, dtype=np.int64)
    if counts.shape != (n,):
        raise ValueError("counts must have one entry per column")
    if counts.max(initial=0) > m:
        raise ValueError("a column cannot hold more nonzeros than there are rows")
    m_eq = m // 2 if m_eq is None else int(m_eq)
    cols, rows = _distinct_rows(rng, counts, m)
    vals = rng.standard_normal(rows.shape[0])
    cp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=cp[1:])
    U = rng.uniform(1.0, 10.0, n)
    x0 = rng.uniform(0.0, U)
    ax0 = np.bincount(rows, weights=vals * x0[cols], minlength=m)
    slack = rng.uniform(0.0, 1.0, m - m_eq)
    y0 = rng.standard_normal(m)
    y0[m_eq:] = -np.abs(y0[m_eq:])
    s = rng.uniform(0.0, 1.0, n)
    c = np.bincount(cols, weights=vals * y0[rows], minlength=n) + s
    row_lower = np.empty(m)
    row_upper = np.empty(m)
    row_lower[:m_eq] = ax0[:m_eq]
    row_upper[:m_eq] = ax0[:m_eq]
    row_lower[m_eq:] = -INF
    row_upper[m_eq:] = ax0[m_eq:] + slack
    rp, ci, rv = csc_to_csr(m, n, cp, rows, vals)
    A = SparseMatrix(m, n, cp, rows, vals, rp, ci, rv)
    return Problem.from_arrays(A, c, np.zeros(n), U, row_lower, row_upper,
                               ObjectiveSense.Minimize, 0.0, name)


def small_random_lp(m: int = 2000, n: int = 5000, nnz_per_col: int = 8, seed: int = 0) -> Problem:
    """m rows (first half equalities, rest <=), n columns, exactly ``nnz_per_col``
    nonzeros per column.  Defaults are the 2,000 x 5,000 / 40k-nnz instance."""
    return random_feasible_lp(m, n, np.full(n, nnz_per_col, dtype=np.int64), seed,
                              name=f"random_{m}x{n}_k{nnz_per_col}_s{seed}")


def zipf_lp(m: int = 500_000, n: int = 1_000_000, nnz: int = 12_000_000, seed: int = 0) -> Problem:
    """Large LP with heavy-tailed column counts: Zipf(1.5) clipped to [2, 2000],
    rescaled to ``nnz`` total.  Defaults are the 500k x 1M / 12M-nnz instance."""
    rng = np.random.default_rng(seed)
    counts = zipf_column_counts(rng, n, nnz)
    return random_feasible_lp(m, n, counts, rng=rng, name=f"zipf_{m}x{n}_nnz{nnz}_s{seed}")


def layer_lp(seed: int, m: int = 20_000, n: int = 50_000, nnz_per_col: int = 10) -> Problem:
    """One instance of the differentiable-layer batch (20k x 50k, 10 nnz/col)."""
    return small_random_lp(m, n, nnz_per_col, seed)

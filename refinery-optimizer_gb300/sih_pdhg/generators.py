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


def mixed_bounds_lp(m: int = 80, n: int = 200, nnz_per_col: int = 4, seed: int = 0) -> Problem:
    """Small LP with every kind of row and column bound, feasible and bounded by
    construction: rows cycle through equality, <=, >=, ranged and free (no
    finite bound), columns through boxed [0, U], lower-only, upper-only, free
    and fixed (lower == upper); the last row and the last column hold no
    nonzeros (the row's bounds [-1, 1] contain its activity 0).  A point x0
    inside the column bounds sets the row bounds around A x0; duals y0 with the
    row types' signs (>= 0 on >= rows, <= 0 on <= rows, 0 on free rows) and a
    reduced cost s with the column types' signs (>= 0 lower-only, <= 0
    upper-only, 0 free) give c = A^T y0 + s, a dual feasible point."""
    rng = np.random.default_rng(seed)
    counts = np.full(n, nnz_per_col, dtype=np.int64)
    counts[-1] = 0
    cols, rows = _distinct_rows(rng, counts, m - 1)  # the last row stays empty
    vals = rng.standard_normal(rows.shape[0])
    cp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=cp[1:])
    ctype = np.arange(n) % 5          # 0 boxed, 1 lower-only, 2 upper-only, 3 free, 4 fixed
    ctype[-1] = 0
    U = rng.uniform(1.0, 10.0, n)
    lo_b = rng.uniform(-2.0, 0.0, n)
    up_b = rng.uniform(0.0, 5.0, n)
    col_lower = np.where(ctype == 0, 0.0, np.where(ctype == 1, lo_b, np.where(ctype == 4, lo_b, -INF)))
    col_upper = np.where(ctype == 0, U, np.where(ctype == 2, up_b, np.where(ctype == 4, lo_b, INF)))
    spread = rng.uniform(0.0, 3.0, n)
    x0 = np.select([ctype == 0, ctype == 1, ctype == 2, ctype == 3, ctype == 4],
                   [rng.uniform(0.0, 1.0, n) * U, lo_b + spread, up_b - spread, rng.normal(0.0, 3.0, n), lo_b])
    ax0 = np.bincount(rows, weights=vals * x0[cols], minlength=m)
    rtype = np.arange(m) % 5          # 0 equality, 1 <=, 2 >=, 3 ranged, 4 free
    rtype[-1] = 3
    gap_lo, gap_up = rng.uniform(0.0, 1.0, m), rng.uniform(0.0, 1.0, m)
    row_lower = np.select([rtype == 0, rtype == 2, rtype == 3], [ax0, ax0 - gap_lo, ax0 - gap_lo], -INF)
    row_upper = np.select([rtype == 0, rtype == 1, rtype == 3], [ax0, ax0 + gap_up, ax0 + gap_up], INF)
    row_lower[-1], row_upper[-1] = -1.0, 1.0
    yn = rng.standard_normal(m)
    y0 = np.select([rtype == 1, rtype == 2, rtype == 4], [-np.abs(yn), np.abs(yn), 0.0], yn)
    sn = rng.standard_normal(n)
    su = rng.uniform(0.0, 1.0, n)
    s = np.select([ctype == 1, ctype == 2, ctype == 3], [su, -su, 0.0], sn)
    c = np.bincount(cols, weights=vals * y0[rows], minlength=n) + s
    rp, ci, rv = csc_to_csr(m, n, cp, rows, vals)
    A = SparseMatrix(m, n, cp, rows, vals, rp, ci, rv)
    return Problem.from_arrays(A, c, col_lower, col_upper, row_lower, row_upper, ObjectiveSense.Minimize, 0.0,
                               f"mixed_bounds_{m}x{n}_s{seed}")

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


# --------------------------------------------------------------------------
# Refinery multi-period planning LP (block-angular, one block per period).
#
# The unit network follows the reference's refinery model
# (py/refinery/model_builder.py:10-57, 143-312: crude purchase, distillation
# cut yields, VDU / FCC / reformer / hydrotreater throughputs and yields,
# blend pools with octane-like and sulphur-like quality rows) and is widened
# to production-planning size: every period has 5 blend pools of 29 product
# grades, each grade with its own blend, 4 quality rows and a product tank.
# Crude tanks and product tanks carry inventory from period t to t + 1, which
# is the only coupling between period blocks.  Minimisation form (cost minus
# revenue); every column is bounded or limited through its rows, and x = 0
# with the tanks at their initial level is feasible, so every instance, with
# or without a unit outage, is feasible and bounded.

REFINERY_POOLS = 5
REFINERY_GRADES = 29
REFINERY_UNITS = ("VDU", "FCC", "REF", "HDT")

# local column layout of the core of a period block
_C_BUY, _C_CINV, _C_FEED, _C_CUT = 0, 3, 6, 9          # 3 crudes, 3 crude tanks, 3 CDU feeds, 6 cuts
_C_VDU, _C_FCC, _C_REF, _C_HDT = 15, 16, 17, 18        # unit throughputs
_C_FCC_FEED, _C_HDT_DIST, _C_HDT_CYC = 19, 20, 21      # internal transfers
_CORE_COLS = 22
# local row layout of the core
_R_CTANK, _R_CDU, _R_CUT, _R_COMP = 0, 3, 4, 10         # 3 crude tanks, CDU capacity, 6 cut yields, 8 components
_R_REF_FEED, _R_VDU_FEED, _R_FCC_FEED, _R_HDT_FEED = 18, 19, 20, 21
_CORE_ROWS = 22
_COMPONENTS = 8   # LPG, light naphtha, reformate, FCC gasoline, raw distillate, HDT distillate, gas oil, residue


def _refinery_template(rng: np.random.Generator):
    """Sparsity template of one period (entries sorted by column, then row).

    Returns (cols, rows, vals, kind, m_per, n_per, grade_layout): ``kind`` is
    -1 for fixed coefficients and 6*c + k for the yield of cut k of crude c
    (drawn per period); rows >= m_per point into the next period's block.
    """
    ent = []  # (col, row, val, kind)

    def add(col, row, val, kind=-1):
        ent.append((col, row, val, kind))

    for c in range(3):
        add(_C_BUY + c, _R_CTANK + c, 1.0)
        add(_C_CINV + c, _R_CTANK + c, -1.0)
        add(_C_FEED + c, _R_CTANK + c, -1.0)
        add(_C_FEED + c, _R_CDU, 1.0)
        for k in range(6):
            add(_C_FEED + c, _R_CUT + k, 0.0, 6 * c + k)
    # cuts: LPG, light naphtha -> components 0, 1; heavy naphtha -> reformer
    # feed; distillate -> component 4; gas oil -> component 6; residue -> VDU
    cut_use = {0: _R_COMP + 0, 1: _R_COMP + 1, 2: _R_REF_FEED, 3: _R_COMP + 4, 4: _R_COMP + 6, 5: _R_VDU_FEED}
    for k in range(6):
        add(_C_CUT + k, _R_CUT + k, 1.0)
        add(_C_CUT + k, cut_use[k], -1.0)
    add(_C_VDU, _R_COMP + 6, -0.6); add(_C_VDU, _R_COMP + 7, -0.4); add(_C_VDU, _R_VDU_FEED, 1.0)
    add(_C_FCC, _R_COMP + 3, -0.55); add(_C_FCC, _R_COMP + 6, -0.3); add(_C_FCC, _R_FCC_FEED, 1.0)
    add(_C_REF, _R_COMP + 2, -0.85); add(_C_REF, _R_REF_FEED, 1.0)
    add(_C_HDT, _R_COMP + 5, -0.98); add(_C_HDT, _R_HDT_FEED, 1.0)
    add(_C_FCC_FEED, _R_COMP + 6, 1.0); add(_C_FCC_FEED, _R_FCC_FEED, -1.0)
    add(_C_HDT_DIST, _R_COMP + 4, 1.0); add(_C_HDT_DIST, _R_HDT_FEED, -1.0)
    add(_C_HDT_CYC, _R_COMP + 6, 1.0); add(_C_HDT_CYC, _R_HDT_FEED, -1.0)

    # component qualities: two octane-like (80..100) and two sulphur-like (0..50 ppm);
    # a quality row is sum_k (q_k - spec) flow_k >= 0 (octane) or <= 0 (sulphur),
    # the form of the reference builder (model_builder.py:271-290)
    octane = rng.uniform(80.0, 100.0, (_COMPONENTS, 2))
    sulphur = rng.uniform(0.0, 50.0, (_COMPONENTS, 2))
    grades = []   # (prod_col, sell_col, inv_col, tank_row)
    col, row = _CORE_COLS, _CORE_ROWS
    for p in range(REFINERY_POOLS):
        allowed = np.sort(rng.choice(_COMPONENTS, size=int(rng.integers(6, 8)), replace=False))
        for g in range(REFINERY_GRADES):
            blend, q0, q1, s0, s1, tank = range(row, row + 6)
            oct_spec = rng.uniform(85.0, 95.0, 2)
            sul_spec = rng.uniform(10.0, 40.0, 2)
            prod, sell, inv = col, col + 1, col + 2
            add(prod, blend, -1.0)
            add(prod, tank, 1.0)
            add(sell, tank, -1.0)
            add(inv, tank, -1.0)
            inv_next = ("next", tank)
            ent.append((inv, inv_next, 1.0, -1))
            for j, k in enumerate(allowed):
                f = col + 3 + j
                add(f, _R_COMP + int(k), 1.0)
                add(f, blend, 1.0)
                add(f, q0, octane[k, 0] - oct_spec[0]); add(f, q1, octane[k, 1] - oct_spec[1])
                add(f, s0, sulphur[k, 0] - sul_spec[0]); add(f, s1, sulphur[k, 1] - sul_spec[1])
            grades.append((prod, sell, inv, tank))
            col += 3 + allowed.shape[0]
            row += 6
    m_per, n_per = row, col
    for c in range(3):  # crude tank of the next period
        ent.append((_C_CINV + c, ("next", _R_CTANK + c), 1.0, -1))
    fixed = [(cc, (m_per + r[1]) if isinstance(r, tuple) else r, v, kd) for cc, r, v, kd in ent]
    arr = np.array([(cc, r, v, kd) for cc, r, v, kd in fixed], dtype=np.float64)
    order = np.lexsort((arr[:, 1], arr[:, 0]))
    arr = arr[order]
    return (arr[:, 0].astype(np.int64), arr[:, 1].astype(np.int64), arr[:, 2], arr[:, 3].astype(np.int64),
            m_per, n_per, np.array(grades, dtype=np.int64))


def refinery_lp(periods: int = 168, seed: int = 0, crude_shock=None, product_shock=None,
                outage_unit: int | None = None, name: str | None = None) -> Problem:
    """Block-angular multi-period refinery planning LP (about 892 rows and
    1,400 columns per period; 168 periods give m = 149,856, n ~ 235k).

    Per period: 3 crude purchases (price ~ U(60, 90)) into crude tanks, one
    CDU whose 6 cut-yield rows use yields ~ U(0.05, 0.35) normalised to sum 1
    (drawn per period and crude), VDU / FCC / reformer / hydrotreater with
    fixed yields and capacities, 8 blend components, 5 pools x 29 grades with
    a blend row, 2 octane-like (>=) and 2 sulphur-like (<=) quality rows and a
    product tank each; product prices ~ U(70, 120).

    ``crude_shock`` (3,) and ``product_shock`` (145,) multiply the crude and
    product prices of every period; ``outage_unit`` in 0..3 (VDU, FCC, REF,
    HDT) zeroes that unit's capacity in every period.
    """
    if periods < 1:
        raise ValueError("periods must be >= 1")
    rng = np.random.default_rng(seed)
    t_col, t_row, t_val, t_kind, m_per, n_per, grades = _refinery_template(rng)
    P = int(periods)
    m, n = P * m_per, P * n_per

    # per-period cut yields (3 crudes x 6 cuts), normalised to sum 1 per crude
    y = rng.uniform(0.05, 0.35, (P, 3, 6))
    y /= y.sum(axis=2, keepdims=True)
    vals = np.broadcast_to(t_val, (P, t_val.shape[0])).copy()
    yk = t_kind >= 0
    vals[:, yk] = -y.reshape(P, 18)[:, t_kind[yk]]

    cols = (np.arange(P, dtype=np.int64)[:, None] * n_per + t_col[None, :]).ravel()
    rows = (np.arange(P, dtype=np.int64)[:, None] * m_per + t_row[None, :]).ravel()
    vals = vals.ravel()
    keep = rows < m   # the last period's tanks link to nothing
    cols, rows, vals = cols[keep], rows[keep], vals[keep]
    cp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(cols, minlength=n), out=cp[1:])

    # costs and bounds
    c = np.zeros((P, n_per))
    lo = np.zeros((P, n_per))
    hi = np.full((P, n_per), INF)
    crude_price = rng.uniform(60.0, 90.0, (P, 3))
    if crude_shock is not None:
        crude_price = crude_price * np.asarray(crude_shock, dtype=np.float64)[None, :]
    c[:, _C_BUY:_C_BUY + 3] = crude_price
    hi[:, _C_BUY:_C_BUY + 3] = rng.uniform(50_000.0, 100_000.0, 3)[None, :]
    c[:, _C_CINV:_C_CINV + 3] = 0.05
    hi[:, _C_CINV:_C_CINV + 3] = 200_000.0
    caps = np.array([50_000.0, 40_000.0, 30_000.0, 45_000.0])
    opcost = rng.uniform(1.0, 5.0, 4)
    if outage_unit is not None:
        caps = caps.copy()
        caps[int(outage_unit)] = 0.0
    for u, cu in enumerate((_C_VDU, _C_FCC, _C_REF, _C_HDT)):
        c[:, cu] = opcost[u]
        hi[:, cu] = caps[u]
    G = grades.shape[0]
    prod_price = rng.uniform(70.0, 120.0, (P, G))
    if product_shock is not None:
        prod_price = prod_price * np.asarray(product_shock, dtype=np.float64)[None, :]
    c[:, grades[:, 1]] = -prod_price
    hi[:, grades[:, 1]] = rng.uniform(2_000.0, 10_000.0, G)[None, :]
    c[:, grades[:, 2]] = 0.05
    hi[:, grades[:, 2]] = 60_000.0

    rl = np.zeros((P, m_per))
    ru = np.zeros((P, m_per))
    ru[:, _R_CDU] = 150_000.0
    rl[:, _R_CDU] = -INF
    rl[:, _R_COMP:_R_COMP + _COMPONENTS] = -INF
    rl[:, _R_REF_FEED:_R_HDT_FEED + 1] = -INF
    for gi in range(G):
        blend = grades[gi, 3] - 5
        ru[:, blend + 1:blend + 3] = INF     # octane-like rows: >= 0
        rl[:, blend + 3:blend + 5] = -INF    # sulphur-like rows: <= 0
    # initial tank levels enter the first period's tank rows
    crude_init = rng.uniform(20_000.0, 60_000.0, 3)
    prod_init = rng.uniform(1_000.0, 10_000.0, G)
    rl[0, _R_CTANK:_R_CTANK + 3] = ru[0, _R_CTANK:_R_CTANK + 3] = -crude_init
    rl[0, grades[:, 3]] = ru[0, grades[:, 3]] = -prod_init

    A = SparseMatrix(m, n, cp, rows, vals)
    nm = name or f"refinery_p{P}_s{seed}"
    return Problem.from_arrays(A, c.ravel(), lo.ravel(), hi.ravel(), rl.ravel(), ru.ravel(),
                               ObjectiveSense.Minimize, 0.0, nm)


def refinery_scenarios(count: int = 512, seed: int = 0, periods_choices=tuple(range(24, 337, 24)),
                       shock_sigma: float = 0.15, outage_fraction: float = 0.10):
    """Price-shock / outage re-solve batch (the reference's scenario
    perturbations, py/refinery/parameterized_generator.py:64-123 and
    py/refinery/reoptimization.py:31-79, at batch scale): scenario s has a
    period count drawn uniformly from ``periods_choices``, its own refinery
    data (seed ``seed * 100003 + s``), crude and product prices multiplied by
    independent lognormal(0, shock_sigma) shocks, and, for a fraction
    ``outage_fraction`` of the scenarios, one unit (VDU, FCC, reformer or
    hydrotreater) out of service in every period."""
    rng = np.random.default_rng(seed)
    G = REFINERY_POOLS * REFINERY_GRADES
    periods = rng.choice(np.asarray(periods_choices), size=count)
    crude = rng.lognormal(0.0, shock_sigma, (count, 3))
    prod = rng.lognormal(0.0, shock_sigma, (count, G))
    n_out = int(round(outage_fraction * count))
    outage = np.full(count, -1)
    outage[rng.choice(count, size=n_out, replace=False)] = rng.integers(0, 4, n_out)
    for s in range(count):
        yield refinery_lp(int(periods[s]), seed * 100003 + s, crude[s], prod[s],
                          None if outage[s] < 0 else int(outage[s]), name=f"refinery_scn{s}_p{periods[s]}")

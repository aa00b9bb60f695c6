"""Every kind of bound (sih_pdhg.generators.mixed_bounds_lp: equality, <=, >=,
ranged and free rows; boxed, lower-only, upper-only, free and fixed columns; an
empty row and an empty column), on the CPU: the generator's LPs are feasible
and bounded (HiGHS finds an optimum), the FP64 oracle of the mixed algorithm
reaches that optimum, and the plain-algorithm oracle (the reference's
arithmetic) runs on them without producing a non-finite value."""
import numpy as np
import pytest

from conftest import highs_general

SEEDS = (0, 1, 2)


def _lp(seed):
    from sih_pdhg.generators import mixed_bounds_lp

    return mixed_bounds_lp(seed=seed)


def test_generator_covers_every_bound_kind():
    p = _lp(0)
    rl, ru, l, u = p.row_lower, p.row_upper, p.col_lower, p.col_upper
    assert np.any(rl == ru)
    assert np.any(~np.isfinite(rl) & np.isfinite(ru)) and np.any(np.isfinite(rl) & ~np.isfinite(ru))
    assert np.any(np.isfinite(rl) & np.isfinite(ru) & (rl < ru))
    assert np.any(~np.isfinite(rl) & ~np.isfinite(ru))
    assert np.any(np.isfinite(l) & ~np.isfinite(u)) and np.any(~np.isfinite(l) & np.isfinite(u))
    assert np.any(~np.isfinite(l) & ~np.isfinite(u)) and np.any(l == u)
    cp, rp = p.A.csc_col_ptr(), p.A.csr_row_ptr()
    assert cp[-1] == cp[-2] and rp[-1] == rp[-2]  # last column and last row hold no nonzeros


@pytest.mark.parametrize("seed", SEEDS)
def test_fp64_oracle_reaches_the_highs_optimum(oracle_lib, seed):
    p = _lp(seed)
    ref, _ = highs_general(p)
    x, y, info = oracle_lib.pdlp_solve(p, tol=1e-8, max_attempts=2_000_000)
    assert info["status"] == 0
    # inside the column bounds up to the rounding of the unscaling (x = x_scaled * d)
    slack = 1e-12 * np.maximum(1.0, np.abs(x))
    assert np.all(x >= p.col_lower - slack) and np.all(x <= p.col_upper + slack)
    assert abs(p.c @ x - ref) <= 1e-7 * max(1.0, abs(ref))
    k = oracle_lib.kkt(p, x, y)
    assert max(k["rel_primal"], k["rel_dual"], k["rel_gap"]) <= 1e-8


@pytest.mark.parametrize("seed", SEEDS)
def test_plain_oracle_stays_finite(oracle_lib, seed):
    import sih_pdhg

    p = _lp(seed)
    x, y, info = oracle_lib.plain_pdhg(p, sih_pdhg.GpuPdhgConfig(max_iterations=20000))
    assert np.isfinite(x).all() and np.isfinite(y).all()
    assert info["status"] in (0, 4)

"""Refinery planning LP generator (block-angular, 168 hourly periods in the
bench) and its scenario batch: sizes, structure, feasibility by
construction, the perturbations, and the FP64 optimum against HiGHS fixtures
(tests/golden/refinery_objectives.json, made by make_refinery_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _fixture():
    with open(os.path.join(GOLDEN, "refinery_objectives.json")) as f:
        return json.load(f)["cases"]


def _build(c):
    from sih_pdhg.generators import refinery_lp

    prod = None if c["product_shock_scale"] is None else np.full(145, c["product_shock_scale"])
    return refinery_lp(c["periods"], c["seed"], c["crude_shock"], prod, c["outage_unit"])


def test_period_block_sizes():
    from sih_pdhg.generators import refinery_lp

    one = refinery_lp(1, 0)
    two = refinery_lp(2, 0)
    assert one.num_rows() == 892 and two.num_rows() == 2 * 892
    assert 1300 <= one.num_cols() <= 1500 and two.num_cols() == 2 * one.num_cols()
    # 168 periods: m = 149,856 and n within the 235k target
    assert refinery_lp(168, 0).num_rows() == 149_856


def test_block_angular_coupling_only_through_tanks():
    from sih_pdhg.generators import refinery_lp

    p = refinery_lp(3, 1)
    mp, npp = p.num_rows() // 3, p.num_cols() // 3
    A = p.A
    cols = np.repeat(np.arange(p.num_cols()), np.diff(A.csc_col_ptr()))
    rows = A.csc_row_ind()
    pc, pr = cols // npp, rows // mp
    assert np.all((pr == pc) | (pr == pc + 1))  # own period, or the next period's tank rows
    link = pr == pc + 1
    assert np.all(A.csc_values()[link] == 1.0)
    # linking entries sit on tank rows: every one is an equality row
    assert np.all(p.row_lower[rows[link]] == p.row_upper[rows[link]])


def test_zero_production_with_full_tanks_is_feasible():
    """x = 0 except the tank inventories held at their initial levels."""
    from sih_pdhg.generators import refinery_lp

    p = refinery_lp(4, 2)
    m, n = p.num_rows(), p.num_cols()
    A = p.A
    # tank inventory columns are the ones with a +1 entry in the next period;
    # their level equals minus the first period's tank row right-hand side
    cols = np.repeat(np.arange(n), np.diff(A.csc_col_ptr()))
    mp, npp = m // 4, n // 4
    link = A.csc_row_ind() // mp == cols // npp + 1
    inv_cols = np.unique(cols[link])
    inv_local = np.unique(inv_cols % npp)
    x = np.zeros(n)
    for j in inv_local:
        k0, k1 = A.csc_col_ptr()[j], A.csc_col_ptr()[j + 1]
        own = A.csc_row_ind()[k0:k1][A.csc_row_ind()[k0:k1] < mp]
        tank_row = own[np.flatnonzero(A.csc_values()[k0:k1][A.csc_row_ind()[k0:k1] < mp] == -1.0)[0]]
        x[j + npp * np.arange(4)] = -p.row_lower[tank_row]
    ax = A.mat_vec(x)
    tol = 1e-6 * (1 + np.abs(ax))
    assert np.all(ax >= p.row_lower - tol) and np.all(ax <= p.row_upper + tol)
    assert np.all(x >= p.col_lower) and np.all(x <= p.col_upper)


def test_scenarios_follow_the_perturbation_recipe():
    from sih_pdhg.generators import REFINERY_UNITS, refinery_scenarios

    probs = list(refinery_scenarios(40, seed=7))
    assert len(probs) == 40
    periods = [p.num_rows() // 892 for p in probs]
    assert set(periods) <= set(range(24, 337, 24))
    # 10% outages: 4 scenarios with a unit capacity column bounded at zero
    outages = 0
    for p, P in zip(probs, periods):
        npp = p.num_cols() // P
        unit_ub = p.col_upper[15:19]  # VDU, FCC, REF, HDT throughputs of period 0
        outages += int(np.any(unit_ub == 0.0))
        assert npp == p.num_cols() // P
    assert outages == 4 and len(REFINERY_UNITS) == 4
    # price shocks: scenarios differ in their objective scale
    assert len({round(float(np.abs(p.c).max()), 6) for p in probs}) > 30


@pytest.mark.parametrize("k", range(5))
def test_highs_objective_fixture(k):
    """The generator is deterministic: HiGHS reproduces the committed optimum."""
    scipy = pytest.importorskip("scipy")
    import sys

    sys.path.insert(0, GOLDEN)
    from make_refinery_golden import highs

    c = _fixture()[k]
    p = _build(c)
    assert (p.num_rows(), p.num_cols(), p.num_nonzeros()) == (c["m"], c["n"], c["nnz"])
    assert abs(highs(p) - c["objective"]) <= 1e-7 * abs(c["objective"])


def test_fp64_oracle_reaches_tolerance_on_a_period_block(oracle_lib):
    import oracle

    c = _fixture()[0]
    p = _build(c)
    x, y, info = oracle.pdlp_solve(p, max_attempts=50000, tol=1e-4)
    assert info["status"] == 0
    assert abs(p.c @ x - c["objective"]) <= 1e-3 * abs(c["objective"])

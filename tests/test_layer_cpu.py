"""Host logic of the LP layer (sih_pdhg.layer), no GPU: which point each
instance returns.  A polished vertex is returned only when the polish
certified its basis optimal; otherwise the instance keeps its PDHG point
(feasible to the solve's tolerance) and is reported."""
from types import SimpleNamespace

import numpy as np
import pytest

from sih_pdhg.layer import choose_outputs


def _info(status=0, pv=0.0, dv=0.0):
    return {"status": status, "primal_violation": pv, "dual_violation": dv}


def test_certified_instances_return_the_vertex_others_the_pdhg_point():
    sols = [SimpleNamespace(x=np.full(3, 10.0 + i), row_duals=np.full(2, -1.0 - i)) for i in range(4)]
    xs = [np.full(3, float(i)) for i in range(4)]
    ys = [np.full(2, float(i)) for i in range(4)]
    infos = [_info(), _info(pv=2e-3), _info(dv=5e-4), _info(status=1)]
    xo, yo, bad = choose_outputs(sols, xs, ys, infos, 1e-6)
    assert bad == [1, 2, 3]
    assert np.array_equal(xo[0], xs[0]) and np.array_equal(yo[0], ys[0])
    for i in bad:
        assert xo[i] is sols[i].x and yo[i] is sols[i].row_duals


def test_certify_tolerance_is_inclusive():
    sols = [SimpleNamespace(x=np.zeros(1), row_duals=np.zeros(1))]
    _, _, bad = choose_outputs(sols, [np.ones(1)], [np.ones(1)], [_info(pv=1e-6, dv=1e-6)], 1e-6)
    assert bad == []


def _highs_with_duals(p):
    """FP64 HiGHS optimum of a minimisation LP whose rows are equalities or <=
    rows: objective, x and the simplex duals (dv/db per row)."""
    sp = pytest.importorskip("scipy.sparse")
    from scipy.optimize import linprog

    A = sp.csc_matrix((p.A.csc_values(), p.A.csc_row_ind(), p.A.csc_col_ptr()), shape=(p.num_rows(), p.num_cols()))
    eq = p.row_lower == p.row_upper
    r = linprog(p.c, A_ub=A[~eq], b_ub=p.row_upper[~eq], A_eq=A[eq], b_eq=p.row_lower[eq],
                bounds=list(zip(p.col_lower, p.col_upper)), method="highs-ds")
    assert r.status == 0
    y = np.zeros(p.num_rows())
    y[eq] = r.eqlin.marginals
    y[~eq] = r.ineqlin.marginals
    return r.fun, r.x, y


def test_objective_gradients_equal_finite_differences_of_the_optimal_value():
    """objective_gradients (the envelope theorem) against central differences of
    FP64 HiGHS re-solves, on the row bounds and the column upper bounds."""
    from sih_pdhg.generators import small_random_lp
    from sih_pdhg.layer import objective_gradients

    p = small_random_lp(40, 100, 4, 3)
    v, x, y = _highs_with_duals(p)
    g = objective_gradients(p, x, -y)
    assert g["objective"] == pytest.approx(v, rel=1e-12)
    h = 1e-4
    rng = np.random.default_rng(0)
    for i in rng.choice(p.num_rows(), 6, replace=False):
        vals = []
        for s in (h, -h):
            q = small_random_lp(40, 100, 4, 3)
            q.row_upper[i] += s
            if q.row_lower[i] == p.row_upper[i]:
                q.row_lower[i] += s  # an equality row moves as a whole
            vals.append(_highs_with_duals(q)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert g["row_lower"][i] + g["row_upper"][i] == pytest.approx(fd, abs=1e-6, rel=1e-6)
    at_upper = np.where(np.isclose(x, p.col_upper))[0]
    for j in at_upper[:6]:
        vals = []
        for s in (h, -h):
            q = small_random_lp(40, 100, 4, 3)
            q.col_upper[j] += s
            vals.append(_highs_with_duals(q)[0])
        assert g["col_upper"][j] == pytest.approx((vals[0] - vals[1]) / (2 * h), abs=1e-6, rel=1e-6)

"""Writes tests/golden/refinery_objectives.json: FP64 optimal objectives of
small refinery planning LPs (sih_pdhg.generators.refinery_lp and the first
scenarios of refinery_scenarios), solved by scipy's HiGHS (dual simplex).

    python tests/golden/make_refinery_golden.py
"""
import json
import os
import sys

import numpy as np
import scipy
import scipy.sparse as sp
from scipy.optimize import linprog

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "refinery-optimizer_gb300"))
from sih_pdhg.generators import refinery_lp  # noqa: E402

CASES = [  # (periods, seed, crude shock, product shock scale, outage unit)
    (1, 0, None, None, None),
    (2, 0, None, None, None),
    (4, 3, None, None, None),
    (3, 5, [1.1, 0.9, 1.2], 0.9, None),
    (3, 5, None, None, 1),  # FCC out of service
]


def highs(p):
    A = sp.csc_matrix((p.A.csc_values(), p.A.csc_row_ind(), p.A.csc_col_ptr()), shape=(p.num_rows(), p.num_cols()))
    eq = p.row_lower == p.row_upper
    ub = (~eq) & (p.row_upper < 1e20)
    lb = (~eq) & (p.row_lower > -1e20)
    A_ub = sp.vstack([A[ub], -A[lb]]).tocsc()
    b_ub = np.concatenate([p.row_upper[ub], -p.row_lower[lb]])
    bounds = list(zip(p.col_lower, [None if u >= 1e20 else u for u in p.col_upper]))
    r = linprog(p.c, A_ub=A_ub, b_ub=b_ub, A_eq=A[eq], b_eq=p.row_lower[eq], bounds=bounds, method="highs-ds")
    assert r.status == 0, r.message
    return float(r.fun)


def build(case):
    P, seed, crude, prod_scale, outage = case
    prod = None if prod_scale is None else np.full(145, prod_scale)
    return refinery_lp(P, seed, crude, prod, outage)


def main():
    out = {"generated_by": f"tests/golden/make_refinery_golden.py (scipy {scipy.__version__}, HiGHS dual simplex)",
           "cases": []}
    for case in CASES:
        p = build(case)
        out["cases"].append({"periods": case[0], "seed": case[1], "crude_shock": case[2],
                             "product_shock_scale": case[3], "outage_unit": case[4], "m": p.num_rows(),
                             "n": p.num_cols(), "nnz": p.num_nonzeros(), "objective": highs(p)})
    with open(os.path.join(HERE, "refinery_objectives.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()

"""Shared test setup: import paths, the ``gpu`` marker and golden-case loaders."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "refinery-optimizer_gb300")
for p in (PKG_DIR, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def golden_index() -> dict:
    with open(os.path.join(GOLDEN, "golden_index.json")) as f:
        return json.load(f)


def golden_case(name: str):
    """(problem, entry, vectors) of one golden case."""
    from sih_pdhg.generators import small_random_lp
    from sih_pdhg.problem import Problem, SparseMatrix

    entry = golden_index()["cases"][name]
    vec = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    if "problem/m" in vec.files:
        A = SparseMatrix(int(vec["problem/m"]), int(vec["problem/n"]), vec["problem/csc_col_ptr"],
                         vec["problem/csc_row_ind"], vec["problem/csc_values"])
        prob = Problem.from_arrays(A, vec["problem/c"], vec["problem/col_lower"], vec["problem/col_upper"],
                                   vec["problem/row_lower"], vec["problem/row_upper"], int(vec["problem/sense"]),
                                   float(vec["problem/obj_offset"]), name)
    else:
        g = entry["generator"]
        prob = small_random_lp(g["m"], g["n"], g["nnz_per_col"], g["seed"])
    return prob, entry, vec


def golden_config(name: str):
    from sih_pdhg.config import GpuPdhgConfig

    cfg = GpuPdhgConfig()
    for k, v in golden_index()["configs"][name].items():
        setattr(cfg, k, v)
    return cfg


def highs_general(problem):
    """FP64 HiGHS (scipy, dual simplex) optimum of a minimisation LP with any mix
    of finite and infinite row and column bounds: (objective, x).  Test oracle only."""
    sp = pytest.importorskip("scipy.sparse")
    from scipy.optimize import linprog

    p = problem
    A = sp.csc_matrix((p.A.csc_values(), p.A.csc_row_ind(), p.A.csc_col_ptr()), shape=(p.num_rows(), p.num_cols()))
    rl, ru = p.row_lower, p.row_upper
    eq = rl == ru
    ub = (~eq) & np.isfinite(ru)
    lb = (~eq) & np.isfinite(rl)
    bounds = [(a if np.isfinite(a) else None, b if np.isfinite(b) else None) for a, b in zip(p.col_lower, p.col_upper)]
    r = linprog(p.c, A_ub=sp.vstack([A[ub], -A[lb]]).tocsc(), b_ub=np.concatenate([ru[ub], -rl[lb]]),
                A_eq=A[eq], b_eq=rl[eq], bounds=bounds, method="highs-ds")
    assert r.status == 0, r.message
    return float(r.fun), r.x


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.lib()
    return oracle

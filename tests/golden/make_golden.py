"""Generate the golden vectors under tests/golden/ from the reference itself.

Run in a container that has the reference sources (default /root/reference)
after ``oracle/ref_build.sh`` has built the reference's pybind module twice
into oracle/_ref/ (see that script).  Writes:

  golden_index.json   scalars of every case (readable summary)
  golden_<case>.npz   vectors of every case

Cases:
  * the LP known answers of the reference's toy suite (data/toy/toy01, toy04,
    toy05; expected objectives and primals from data/toy/toy_suite_metadata.json)
    with the problem arrays as the reference's MPS reader produces them;
  * seeded random feasible LPs from sih_pdhg.generators (the problem itself is
    pinned by a SHA-256 of its arrays, small ones are also stored).
For each case it records:
  * the reference GPU PDHG driver + kernels run on the CPU with the intended
    int32 index copy (``GpuSolver.solve_pdhg``, gpu_solver.cpp:60-307), under
    several GpuPdhgConfig settings: status, iteration count, best x, last y,
    objective;
  * the same with the shipped byte-for-byte index copy (status and objective
    only, to document the shipped defect), default config;
  * the reference FP64 dual simplex (``SimplexSolver::solve``,
    simplex_solver.cpp:92) where it finishes in seconds;
  * scipy's HiGHS (test oracle, as tests/oracle/highs_oracle.py in the
    reference) objective, x and row duals.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "refinery-optimizer_gb300"))

REF_DIR = os.environ.get("SIH_REFERENCE_DIR", "/root/reference")
TOYS = ["toy01_lp_simple", "toy04_lp_equality_ranges", "toy05_lp_bounds"]
RANDOM = [  # (tag, m, n, k, seed, store_arrays, run_simplex)
    ("rand_50x120_k4_s1", 50, 120, 4, 1, True, True),
    ("rand_100x250_k6_s0", 100, 250, 6, 0, True, True),
    ("rand_200x500_k8_s0", 200, 500, 8, 0, True, False),
    ("rand_2000x5000_k8_s0", 2000, 5000, 8, 0, False, False),
]
CONFIGS = {
    "default": {},
    "long": {"max_iterations": 8000},
    "fixed_steps": {"max_iterations": 3000, "check_frequency": 10, "step_tau": 0.05, "step_sigma": 0.05,
                    "enable_restart": False},
    "gpu_basic": {"max_iterations": 2000, "tol_primal": 1e-4},  # tests/test_gpu_basic.py:44-46
}


def problem_digest(p) -> str:
    h = hashlib.sha256()
    A = p.A
    for a in (A.csc_col_ptr(), A.csc_row_ind(), A.csc_values(), p.c, p.col_lower, p.col_upper, p.row_lower,
              p.row_upper):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def problem_arrays(p) -> dict:
    A = p.A
    return dict(m=p.num_rows(), n=p.num_cols(), csc_col_ptr=A.csc_col_ptr(), csc_row_ind=A.csc_row_ind(),
                csc_values=A.csc_values(), c=p.c, col_lower=p.col_lower, col_upper=p.col_upper,
                row_lower=p.row_lower, row_upper=p.row_upper, sense=int(p.sense), obj_offset=p.obj_offset)


# --------------------------------------------------------------------------- reference side (subprocess)
def _ref_child(variant: str, spec_path: str, out_path: str) -> None:
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref", variant))
    import _core  # the reference's pybind module built by oracle/ref_build.sh

    spec = np.load(spec_path, allow_pickle=True)
    cases = json.loads(str(spec["cases"]))
    results = {}
    for case in cases:
        if case["kind"] == "toy":
            prob = _core.read_mps(os.path.join(REF_DIR, "data", "toy", case["name"] + ".mps"))
            A = prob.A
            results[case["name"] + "/problem"] = dict(
                m=prob.num_rows(), n=prob.num_cols(), csc_col_ptr=np.array(A.csc_col_ptr(), np.int64),
                csc_row_ind=np.array(A.csc_row_ind(), np.int64), csc_values=np.array(A.csc_values()),
                c=np.array(prob.c), col_lower=np.array(prob.col_lower), col_upper=np.array(prob.col_upper),
                row_lower=np.array(prob.row_lower), row_upper=np.array(prob.row_upper),
                sense=int(prob.sense.value), obj_offset=prob.obj_offset)
        else:
            d = np.load(case["arrays"])
            m, n = int(d["m"]), int(d["n"])
            prob = _core.Problem(case["name"])
            prob.resize(m, n)
            cp, ri, cv = d["csc_col_ptr"], d["csc_row_ind"], d["csc_values"]
            cols = np.repeat(np.arange(n), np.diff(cp))
            trips = [_core.Triplet(int(r), int(c), float(v)) for r, c, v in zip(ri, cols, cv)]
            prob.A = _core.SparseMatrix.from_triplets(m, n, trips)
            prob.c = d["c"].tolist()
            prob.col_lower = d["col_lower"].tolist()
            prob.col_upper = d["col_upper"].tolist()
            prob.row_lower = d["row_lower"].tolist()
            prob.row_upper = d["row_upper"].tolist()
        for cname in case["configs"]:
            cfg = _core.GpuPdhgConfig()
            for k, v in CONFIGS[cname].items():
                setattr(cfg, k, v)
            sol = _core.GpuSolver.solve_pdhg(prob, cfg)
            results[f"{case['name']}/pdhg/{cname}"] = dict(
                status=int(sol.status.value), iterations=int(sol.simplex_iterations), x=np.array(sol.x),
                row_duals=np.array(sol.row_duals), primal_objective=sol.primal_objective)
        if case.get("simplex"):
            o = _core.Options()
            o.strategy.algorithm = _core.AlgorithmChoice.DualSimplex
            sol = _core.SimplexSolver.solve(prob, o)
            results[f"{case['name']}/simplex"] = dict(
                status=int(sol.status.value), x=np.array(sol.x), row_duals=np.array(sol.row_duals),
                primal_objective=sol.primal_objective)
    flat = {}
    for key, val in results.items():
        for k2, v2 in val.items():
            flat[f"{key}/{k2}"] = np.asarray(v2)
    np.savez(out_path, **flat)


def run_reference(variant: str, cases: list) -> dict:
    spec = os.path.join(REPO, "oracle", "_ref", f"spec_{variant}.npz")
    out = os.path.join(REPO, "oracle", "_ref", f"out_{variant}.npz")
    np.savez(spec, cases=json.dumps(cases))
    subprocess.check_call([sys.executable, os.path.abspath(__file__), "--child", variant, spec, out])
    d = np.load(out)
    return {k: d[k] for k in d.files}


# --------------------------------------------------------------------------- HiGHS (scipy)
def highs(prob) -> dict:
    from scipy.optimize import linprog
    from scipy.sparse import csc_matrix

    A = prob.A
    M = csc_matrix((A.csc_values(), A.csc_row_ind(), A.csc_col_ptr()), shape=(prob.num_rows(), prob.num_cols()))
    rl, ru = prob.row_lower, prob.row_upper
    eq = rl == ru
    ub_hi = (~eq) & np.isfinite(ru)
    ub_lo = (~eq) & np.isfinite(rl)
    import scipy.sparse as sp
    A_ub = sp.vstack([M[ub_hi], -M[ub_lo]]).tocsr()
    b_ub = np.concatenate([ru[ub_hi], -rl[ub_lo]])
    bounds = list(zip(np.where(np.isfinite(prob.col_lower), prob.col_lower, None),
                      np.where(np.isfinite(prob.col_upper), prob.col_upper, None)))
    c = prob.c * (1 if int(prob.sense) == 1 else -1)
    res = linprog(c, A_ub=A_ub if A_ub.shape[0] else None, b_ub=b_ub if A_ub.shape[0] else None,
                  A_eq=M[eq] if eq.any() else None, b_eq=rl[eq] if eq.any() else None, bounds=bounds,
                  method="highs-ipm")
    assert res.status == 0, res.message
    y = np.zeros(prob.num_rows())  # simplex sign: d obj / d b
    if eq.any():
        y[eq] = res.eqlin.marginals
    if A_ub.shape[0]:
        mu = res.ineqlin.marginals
        nh = int(ub_hi.sum())
        y[ub_hi] += mu[:nh]
        y[ub_lo] -= mu[nh:]
    obj = res.fun * (1 if int(prob.sense) == 1 else -1) + prob.obj_offset
    return dict(objective=float(obj), x=res.x, row_duals=y)


def main() -> None:
    from sih_pdhg.generators import small_random_lp
    from sih_pdhg.problem import Problem, SparseMatrix

    meta = json.load(open(os.path.join(REF_DIR, "data", "toy", "toy_suite_metadata.json")))
    expected = {p["name"]: p for p in meta["problems"]}
    cases = [dict(kind="toy", name=t, configs=list(CONFIGS), simplex=True) for t in TOYS]
    gens = {}
    for tag, m, n, k, seed, store, simplex in RANDOM:
        p = small_random_lp(m, n, k, seed)
        gens[tag] = (p, store, (m, n, k, seed))
        arr_path = os.path.join(REPO, "oracle", "_ref", f"problem_{tag}.npz")
        np.savez(arr_path, **problem_arrays(p))
        cases.append(dict(kind="random", name=tag, arrays=arr_path, configs=list(CONFIGS), simplex=simplex))

    intended = run_reference("intended", cases)
    faithful = run_reference("faithful", [dict(c, configs=["default"], simplex=False) for c in cases])

    index = {"generated_by": "tests/golden/make_golden.py", "configs": CONFIGS, "cases": {}}
    for case in cases:
        name = case["name"]
        vec = {}
        entry = {"kind": case["kind"]}
        if case["kind"] == "toy":
            pre = f"{name}/problem/"
            pa = {k[len(pre):]: intended[k] for k in intended if k.startswith(pre)}
            for k, v in pa.items():
                vec["problem/" + k] = v
            A = SparseMatrix(int(pa["m"]), int(pa["n"]), pa["csc_col_ptr"], pa["csc_row_ind"], pa["csc_values"])
            prob = Problem.from_arrays(A, pa["c"], pa["col_lower"], pa["col_upper"], pa["row_lower"],
                                       pa["row_upper"], int(pa["sense"]), float(pa["obj_offset"]), name)
            entry["expected_objective"] = expected[name]["expected_objective"]
            entry["expected_primal"] = expected[name]["expected_primal"]
        else:
            prob, store, (m, n, k, seed) = gens[name]
            entry["generator"] = dict(fn="small_random_lp", m=m, n=n, nnz_per_col=k, seed=seed)
            entry["sha256"] = problem_digest(prob)
            if store:
                for kk, v in problem_arrays(prob).items():
                    vec["problem/" + kk] = np.asarray(v)
        entry["pdhg"] = {}
        for cname in case["configs"]:
            pre = f"{name}/pdhg/{cname}/"
            entry["pdhg"][cname] = dict(status=int(intended[pre + "status"]),
                                        iterations=int(intended[pre + "iterations"]),
                                        primal_objective=float(intended[pre + "primal_objective"]))
            vec[f"pdhg/{cname}/x"] = intended[pre + "x"]
            vec[f"pdhg/{cname}/row_duals"] = intended[pre + "row_duals"]
        pre = f"{name}/pdhg/default/"
        entry["shipped_index_copy"] = dict(status=int(faithful[pre + "status"]),
                                           iterations=int(faithful[pre + "iterations"]),
                                           primal_objective=float(faithful[pre + "primal_objective"]))
        if case.get("simplex"):
            pre = f"{name}/simplex/"
            entry["simplex"] = dict(status=int(intended[pre + "status"]),
                                    primal_objective=float(intended[pre + "primal_objective"]))
            vec["simplex/x"] = intended[pre + "x"]
            vec["simplex/row_duals"] = intended[pre + "row_duals"]
        h = highs(prob)
        entry["highs_objective"] = h["objective"]
        vec["highs/x"] = h["x"]
        vec["highs/row_duals"] = h["row_duals"]
        np.savez_compressed(os.path.join(HERE, f"golden_{name}.npz"), **vec)
        index["cases"][name] = entry
        print(name, json.dumps({k: v for k, v in entry.items() if k in ("pdhg", "simplex", "highs_objective")}))
    with open(os.path.join(HERE, "golden_index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--child":
        _ref_child(sys.argv[2], sys.argv[3], sys.argv[4])
    else:
        main()

"""Times the reference's own FP64 solvers on the LP generator's ladder, for the
CPU-baseline table of the engine's design notes (reference dual simplex:
sih_solver SimplexSolver::solve, core/src/simplex/simplex_solver.cpp:92; and
scipy's HiGHS interior point, the FP64 objective oracle of the tests).

Needs the reference build of oracle/ref_build.sh (oracle/_ref/intended), so it
runs only where the reference sources are present:

    python oracle/time_reference_solvers.py [--limit SECONDS]

Each solve runs in a child process killed at the limit ("did not finish").
Timings are of this host, one solve at a time.
"""
import argparse
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "refinery-optimizer_gb300"))

LADDER = [(100, 250, 8), (200, 500, 8), (400, 1000, 8), (2000, 5000, 8)]
HIGHS = [(2000, 5000, 8), (20000, 50000, 10)]

SIMPLEX_CHILD = """
import sys, time
sys.path.insert(0, {core!r})
import _core
p = _core.read_mps({path!r})
o = _core.Options()
o.strategy.algorithm = _core.AlgorithmChoice.DualSimplex
t = time.perf_counter()
s = _core.SimplexSolver.solve(p, o)
print("RESULT", time.perf_counter() - t, s.status, repr(s.primal_objective))
"""

HIGHS_CHILD = """
import sys, time
sys.path.insert(0, {pkg!r})
import numpy as np, scipy.sparse as sp
from scipy.optimize import linprog
import sih_pdhg
p = sih_pdhg.read_mps({path!r})
A = sp.csc_matrix((p.A.csc_values(), p.A.csc_row_ind(), p.A.csc_col_ptr()), shape=(p.num_rows(), p.num_cols()))
rl, ru = p.row_lower, p.row_upper
eq = rl == ru; ub = (~eq) & np.isfinite(ru); lb = (~eq) & np.isfinite(rl)
t = time.perf_counter()
r = linprog(p.c, A_ub=sp.vstack([A[ub], -A[lb]]).tocsc(), b_ub=np.concatenate([ru[ub], -rl[lb]]), A_eq=A[eq],
            b_eq=rl[eq], bounds=list(zip(p.col_lower, p.col_upper)), method="highs-ipm")
print("RESULT", time.perf_counter() - t, r.status, repr(r.fun))
"""


def run(code, limit):
    t = time.perf_counter()
    try:
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=limit)
    except subprocess.TimeoutExpired:
        return f"did not finish in {limit:.0f} s"
    for line in r.stdout.splitlines():
        if line.startswith("RESULT"):
            _, secs, status, obj = line.split(" ", 3)
            return f"{float(secs):.2f} s (status {status}, objective {float(obj):.10g})"
    return f"failed after {time.perf_counter() - t:.1f} s: {r.stderr.strip().splitlines()[-1:]}"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--limit", type=float, default=300.0)
    args = ap.parse_args()
    import sih_pdhg
    from sih_pdhg.generators import small_random_lp

    core = os.path.join(HERE, "_ref", "intended")
    with tempfile.TemporaryDirectory() as tmp:
        print("| LP (generator of the 2,000 x 5,000 workload) | solver | time |")
        print("|---|---|---|")
        for m, n, k in LADDER:
            path = os.path.join(tmp, f"r{m}.mps")
            sih_pdhg.write_mps(small_random_lp(m, n, k, 0), path)
            res = run(SIMPLEX_CHILD.format(core=core, path=path), args.limit)
            print(f"| {m} x {n}, {k}/col | reference dual simplex | {res} |", flush=True)
        for m, n, k in HIGHS:
            path = os.path.join(tmp, f"h{m}.mps")
            sih_pdhg.write_mps(small_random_lp(m, n, k, 0), path)
            res = run(HIGHS_CHILD.format(pkg=os.path.join(REPO, "refinery-optimizer_gb300"), path=path), args.limit)
            print(f"| {m} x {n}, {k}/col | scipy HiGHS IPM | {res} |", flush=True)


if __name__ == "__main__":
    main()

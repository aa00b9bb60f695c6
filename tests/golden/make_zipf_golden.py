"""FP64 oracle results for the Zipf parity case (tests/test_zipf_gpu.py).

    python tests/golden/make_zipf_golden.py     # about 20 minutes on 8 cores (1e-8: 267k steps)

The LP is sih_pdhg.generators.zipf_lp(100_000, 200_000, 2_400_000, seed=1): the
generator of the 500,000 x 1,000,000 benchmark LP (column counts Zipf(1.5)
clipped to [2, 2000], rescaled to the nonzero total) at a fifth of its size.
The oracle is oracle/pdlp_oracle.c, the FP64 restatement of the mixed
algorithm, run to relative KKT 1e-4 and 1e-6 (iterations, restarts, objective)
and to 1e-8 (a sharper objective to compare 1e-6 solves with).  Writes
tests/golden/zipf_100kx200k_s1.json.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "refinery-optimizer_gb300"), os.path.join(REPO, "oracle")]

CASE = {"m": 100_000, "n": 200_000, "nnz": 2_400_000, "seed": 1}


def problem_summary(p) -> dict:
    """Sizes and coarse sums of the LP's arrays (they pin the generator's output
    to a few parts in 1e9, whatever the last bits of its floating point)."""
    A = p.A
    return {"nnz": int(p.num_nonzeros()), "sum_abs_values": float(np.abs(A.csc_values()).sum()),
            "sum_c": float(p.c.sum()), "sum_col_upper": float(p.col_upper.sum()),
            "sum_row_upper_finite": float(p.row_upper[np.isfinite(p.row_upper)].sum()),
            "max_col_nnz": int(np.diff(A.csc_col_ptr()).max())}


def main() -> None:
    import oracle
    from sih_pdhg.generators import zipf_lp

    oracle.build()
    p = zipf_lp(CASE["m"], CASE["n"], CASE["nnz"], CASE["seed"])
    out = {"case": CASE, "problem": problem_summary(p), "oracle": {}}
    for tol in (1e-4, 1e-6, 1e-8):
        t0 = time.perf_counter()
        _, _, info = oracle.pdlp_solve(p, tol=tol, max_attempts=400_000)
        dt = time.perf_counter() - t0
        out["oracle"][f"{tol:g}"] = {k: info[k] for k in ("attempts", "steps", "restarts", "rel_p", "rel_d", "rel_g",
                                                            "pobj", "dobj")}
        out["oracle"][f"{tol:g}"]["seconds"] = round(dt, 1)
        print(tol, out["oracle"][f"{tol:g}"], flush=True)
    with open(os.path.join(HERE, "zipf_100kx200k_s1.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()

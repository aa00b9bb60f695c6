"""FP64 optimal duals of four differentiable-layer LPs (tests/test_layer_gpu.py).

    python tests/golden/make_layer_duals.py     # about 25 minutes on 8 cores (210k-315k steps each)

The LPs are sih_pdhg.generators.layer_lp(seed) for seeds 0..3: the random
feasible generator at 20,000 rows x 50,000 columns, 10 nonzeros per column,
the size of the differentiable-layer batch.  Their duals come from the FP64
oracle (oracle/pdlp_oracle.c, the FP64 restatement of the mixed algorithm) run
to relative KKT 1e-9; by the envelope theorem they are the gradient of the
optimal value with respect to the row bounds (d obj / d b = y*, simplex sign).
scipy's HiGHS interior point did not finish one such LP in 15 minutes on this
container's host (its normal-equation factor fills in), so the oracle at 1e-9
stands in for an FP64 simplex here.  Writes tests/golden/layer_duals.npz
(float32 duals, float64 objectives and the oracle's KKT).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "refinery-optimizer_gb300"), os.path.join(REPO, "oracle")]

SEEDS = (0, 1, 2, 3)


def main() -> None:
    import oracle
    from sih_pdhg.generators import layer_lp

    oracle.build()
    out = {}
    for s in SEEDS:
        p = layer_lp(s)
        t0 = time.perf_counter()
        x, y_pdhg, info = oracle.pdlp_solve(p, tol=1e-9, max_attempts=2_000_000)
        dt = time.perf_counter() - t0
        out[f"y{s}"] = (-y_pdhg).astype(np.float32)  # simplex sign: d obj / d b
        out[f"obj{s}"] = np.float64(info["pobj"])
        out[f"kkt{s}"] = np.array([info["rel_p"], info["rel_d"], info["rel_g"]])
        out[f"attempts{s}"] = np.int64(info["attempts"])
        print(f"seed {s}: {info['attempts']} steps, {dt:.0f} s, KKT {out[f'kkt{s}']}, obj {info['pobj']:.10g}",
              flush=True)
    np.savez_compressed(os.path.join(HERE, "layer_duals.npz"), **out)


if __name__ == "__main__":
    main()

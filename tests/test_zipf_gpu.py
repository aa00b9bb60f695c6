"""Mixed path against the FP64 oracle on a Zipf LP near the benchmark's scale:
zipf_lp(100,000, 200,000, 2.4M nonzeros, seed 1), the 500,000 x 1,000,000
benchmark generator at a fifth of its size (heavy columns up to a few hundred
nonzeros).  The oracle's results (oracle/pdlp_oracle.c in FP64, to relative
KKT 1e-4, 1e-6 and 1e-8) are the fixture tests/golden/zipf_100kx200k_s1.json,
written by tests/golden/make_zipf_golden.py."""
import json
import os
import sys

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


@pytest.fixture(scope="module")
def case():
    sys.path.insert(0, GOLDEN)
    from make_zipf_golden import problem_summary
    from sih_pdhg.generators import zipf_lp

    with open(os.path.join(GOLDEN, "zipf_100kx200k_s1.json")) as f:
        fx = json.load(f)
    c = fx["case"]
    p = zipf_lp(c["m"], c["n"], c["nnz"], c["seed"])
    got = problem_summary(p)
    for k, v in fx["problem"].items():  # the same LP as the oracle solved
        assert got[k] == pytest.approx(v, rel=1e-9), k
    return p, fx


@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_zipf_mixed_solve_matches_fp64_oracle(sih, case, tol):
    p, fx = case
    cfg = sih.GpuPdhgConfig(max_iterations=400_000, tol_primal=tol, tol_dual=tol, tol_gap=tol)
    s = sih.solve_gpu_mixed(p, cfg)
    o = fx["oracle"][f"{tol:g}"]
    ref = fx["oracle"]["1e-08"]["pobj"]  # objective of the FP64 oracle at 1e-8
    print(f"tol {tol:g}: GPU {s.simplex_iterations} steps, {s.restarts} restarts, KKT "
          f"({s.rel_primal:.2e}, {s.rel_dual:.2e}, {s.rel_gap:.2e}), obj {s.primal_objective:.9g}; "
          f"oracle {o['attempts']} steps, {o['restarts']} restarts, obj {o['pobj']:.9g}; 1e-8 obj {ref:.9g}")
    assert s.is_optimal()
    # the solver stopped on its device FP64 test; the host FP64 KKT of the
    # returned point (original space) agrees with it
    assert max(s.rel_primal, s.rel_dual, s.rel_gap) <= 2 * tol
    # objective: within the gap tolerance of the oracle's 1e-8 optimum
    assert abs(s.primal_objective - ref) <= 2 * tol * (1 + 2 * abs(ref))
    # work: FP32 iterates follow the FP64 method's trajectory to within a
    # third of its step count
    assert abs(s.simplex_iterations - o["attempts"]) <= max(3 * 64, 0.35 * o["attempts"])

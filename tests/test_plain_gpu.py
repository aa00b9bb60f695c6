"""GPU parity of the plain (reference-semantics) FP32 PDHG path, through the C ABI.

Oracle: the C restatement in oracle/pdhg_oracle.c, itself pinned bit for bit
to the reference's own driver and kernels (tests/test_oracle_golden.py).
  * exact_arithmetic=1: the GPU result equals the golden vectors bit for bit
    (same iteration count, same best x, same y);
  * default fast SpMV (warp groups + FMA): the same termination within one
    check period (25 iterations) and the objective within 1e-5 relative.
"""
import numpy as np
import pytest

from conftest import golden_case, golden_config, golden_index

pytestmark = pytest.mark.gpu

CASES = [(name, cname) for name, e in sorted(golden_index()["cases"].items()) for cname in sorted(e["pdhg"])]


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


@pytest.mark.parametrize("name,cname", CASES)
def test_exact_mode_bit_identical_to_reference(sih, name, cname):
    prob, entry, vec = golden_case(name)
    ref = entry["pdhg"][cname]
    sol = sih.GpuSolver.solve_ex(prob, golden_config(cname), algorithm=sih.ALGO_PLAIN, exact_arithmetic=1)
    assert int(sol.status) == ref["status"]
    assert sol.simplex_iterations == ref["iterations"]
    np.testing.assert_array_equal(sol.x, vec[f"pdhg/{cname}/x"])
    np.testing.assert_array_equal(sol.row_duals, vec[f"pdhg/{cname}/row_duals"])
    assert sol.primal_objective == pytest.approx(ref["primal_objective"], rel=1e-13, abs=1e-13)


@pytest.mark.parametrize("name,cname", CASES)
def test_fast_mode_matches_reference(sih, name, cname):
    prob, entry, vec = golden_case(name)
    cfg = golden_config(cname)
    ref = entry["pdhg"][cname]
    sol = sih.solve_gpu_pdhg(prob, cfg)
    if ref["status"] == 0:
        assert sol.status == sih.SolutionStatus.Optimal
        assert abs(sol.simplex_iterations - ref["iterations"]) <= cfg.check_frequency
        assert sol.ref_primal <= cfg.tol_primal and sol.ref_dual <= cfg.tol_dual
    else:
        # both run to the cap; the reference reports max_iterations + 1
        assert sol.simplex_iterations in (ref["iterations"], ref["iterations"] - 1 - (cfg.max_iterations % cfg.check_frequency))
    assert sol.primal_objective == pytest.approx(ref["primal_objective"], rel=1e-5, abs=1e-5)
    np.testing.assert_allclose(sol.x, vec[f"pdhg/{cname}/x"], atol=2e-3 * max(1.0, np.abs(sol.x).max()))


def test_toy_known_answers(sih):
    """data/toy/toy_suite_metadata.json expected objectives (toy01, toy04, toy05)."""
    for name, e in golden_index()["cases"].items():
        if e["kind"] != "toy":
            continue
        prob, entry, _ = golden_case(name)
        sol = sih.solve_gpu_pdhg(prob)
        assert sol.is_optimal()
        assert sol.primal_objective == pytest.approx(entry["expected_objective"], rel=1e-4, abs=1e-4)
        np.testing.assert_allclose(sol.x, entry["expected_primal"], atol=2e-3)


def test_objective_vs_fp64_simplex(sih):
    """Converged plain PDHG objective vs the reference dual simplex / HiGHS (FP64)."""
    for name in ("rand_50x120_k4_s1", "rand_100x250_k6_s0", "rand_2000x5000_k8_s0"):
        prob, entry, _ = golden_case(name)
        sol = sih.solve_gpu_pdhg(prob, sih.GpuPdhgConfig(max_iterations=20000))
        assert sol.is_optimal()
        assert sol.primal_objective == pytest.approx(entry["highs_objective"], rel=1e-3)
        assert sol.rel_primal < 1e-3 and sol.rel_gap < 1e-2


def test_empty_problem_is_optimal(sih):
    from sih_pdhg.problem import Problem, SparseMatrix

    A = SparseMatrix(0, 3, np.zeros(4, np.int64), np.zeros(0, np.int64), np.zeros(0))
    p = Problem.from_arrays(A, np.ones(3), np.zeros(3), np.ones(3), np.zeros(0), np.zeros(0))
    sol = sih.solve_gpu_pdhg(p)
    assert sol.status == sih.SolutionStatus.Optimal


def test_maximize_and_offset(sih):
    """Sense and objective offset are honoured (the reference ignores both, gpu_solver.cpp:300-302)."""
    prob, entry, _ = golden_case("toy01_lp_simple")
    prob.sense = sih.ObjectiveSense.Maximize
    prob.c = -prob.c
    prob.obj_offset = 3.0
    sol = sih.solve_gpu_pdhg(prob)
    assert sol.is_optimal()
    assert sol.primal_objective == pytest.approx(6.5 + 3.0, rel=1e-4)


def test_vram_info(sih):
    info = sih.GpuSolver.get_vram_info()
    assert info.total_bytes > 1 << 30 and info.free_bytes <= info.total_bytes

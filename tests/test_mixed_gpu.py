"""GPU parity of the mixed-precision restarted adaptive PDHG (FP32 SpMV, FP64
reductions) against its FP64 oracle (oracle/pdlp_oracle.c), through the C ABI.

* trajectory: after the same number of steps the controller made the same
  decisions (attempts, accepted steps, rejections, restarts) and the step size,
  primal weight and returned point agree to FP32 accuracy (1e-3 relative);
* full solves: the relative KKT error (recomputed on the host in FP64 from the
  original data) meets the tolerance (1e-4 and 1e-6) and the objective matches
  the FP64 simplex/HiGHS objective of the golden vectors.
"""
import numpy as np
import pytest

from conftest import golden_case, golden_index

pytestmark = pytest.mark.gpu
NAMES = sorted(golden_index()["cases"])


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


# The oracle runs with the CUDA path's precision layout (fp32_bits=27: FP32 data,
# iterates and products, FP64 averages with FP32 candidates).
FP32_LAYOUT = 27


@pytest.mark.parametrize("name", ["rand_50x120_k4_s1", "rand_200x500_k8_s0", "rand_2000x5000_k8_s0"])
@pytest.mark.parametrize("blocks", [1, 3])
def test_trajectory_matches_oracle(sih, oracle_lib, name, blocks):
    prob, _, _ = golden_case(name)
    its = 64 * blocks
    cfg = sih.GpuPdhgConfig(max_iterations=its, tol_primal=1e-12, tol_dual=1e-12, tol_gap=1e-12)
    sol = sih.solve_gpu_mixed(prob, cfg, compensated=0)
    x, y, info = oracle_lib.pdlp_solve(prob, max_attempts=its, tol=1e-12, fp32_bits=FP32_LAYOUT)
    assert sol.status == sih.SolutionStatus.IterationLimit and info["status"] == 4
    assert sol.simplex_iterations == info["attempts"]
    assert sol.restarts == info["restarts"]
    assert sol.step_rejections == info["rejections"]
    sx = max(1.0, np.abs(x).max())
    sy = max(1.0, np.abs(y).max())
    np.testing.assert_allclose(sol.x, x, atol=1e-2 * sx)
    np.testing.assert_allclose(sol.row_duals, y, atol=1e-2 * sy)
    # the step size is a ratio of small differences of FP32 iterates, so it drifts
    # from the oracle's with every accepted step: 2 % after one evaluation
    # period; after several only its magnitude is pinned (factor 2)
    if blocks == 1:
        assert sol.final_step == pytest.approx(info["eta"], rel=2e-2)
        assert sol.final_primal_weight == pytest.approx(info["omega"], rel=2e-2)
    else:
        assert 0.5 < sol.final_step / info["eta"] < 2.0
        assert 0.5 < sol.final_primal_weight / info["omega"] < 2.0


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_solves_to_tolerance(sih, oracle_lib, name, tol):
    prob, entry, _ = golden_case(name)
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=tol, tol_dual=tol, tol_gap=tol)
    sol = sih.solve_gpu_mixed(prob, cfg)
    assert sol.status == sih.SolutionStatus.Optimal
    # FP64 host recheck of the returned point on the original data
    assert sol.rel_primal <= 2 * tol and sol.rel_dual <= 2 * tol and sol.rel_gap <= 2 * tol
    k = oracle_lib.kkt(prob, sol.x, sol.row_duals)
    assert k["rel_primal"] == pytest.approx(sol.rel_primal, rel=1e-6, abs=1e-12)
    ref = entry["highs_objective"]
    assert abs(sol.primal_objective - ref) <= 40 * tol * (1 + abs(ref))
    _, _, info = oracle_lib.pdlp_solve(prob, tol=tol, fp32_bits=FP32_LAYOUT)
    # same algorithm, same termination test: within a few evaluation periods of the
    # oracle at 1e-4; within a factor 2 at 1e-6, where FP32 rounding steers the path
    slack = max(4 * 64, 0.25 * info["attempts"]) if tol >= 1e-4 else max(8 * 64, 1.0 * info["attempts"])
    assert abs(sol.simplex_iterations - info["attempts"]) <= slack


def test_simplex_sign_duals(sih):
    """dual_sign=1 returns the simplex convention (row_duals = -y_pdhg), as HiGHS marginals."""
    prob, entry, vec = golden_case("rand_200x500_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    sol = sih.solve_gpu_mixed(prob, cfg, dual_sign=1)
    np.testing.assert_allclose(sol.row_duals, vec["highs/row_duals"], atol=5e-3 * max(1, np.abs(vec["highs/row_duals"]).max()))


def test_maximize(sih):
    prob, entry, _ = golden_case("toy01_lp_simple")
    prob.sense = sih.ObjectiveSense.Maximize
    prob.c = -prob.c
    cfg = sih.GpuPdhgConfig(max_iterations=100000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    sol = sih.solve_gpu_mixed(prob, cfg)
    assert sol.is_optimal()
    assert sol.primal_objective == pytest.approx(6.5, rel=1e-4)


def test_iteration_limit_status(sih):
    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    sol = sih.solve_gpu_mixed(prob, sih.GpuPdhgConfig(max_iterations=128, tol_primal=1e-9, tol_dual=1e-9, tol_gap=1e-9))
    assert sol.status == sih.SolutionStatus.IterationLimit
    assert sol.simplex_iterations == 128


def test_tile_size_does_not_change_decisions(sih):
    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=1e-4, tol_dual=1e-4, tol_gap=1e-4)
    a = sih.solve_gpu_mixed(prob, cfg, tile_nnz=512)
    b = sih.solve_gpu_mixed(prob, cfg, tile_nnz=4096)
    assert a.is_optimal() and b.is_optimal()
    assert abs(a.simplex_iterations - b.simplex_iterations) <= 2 * 64


def test_renumbering_does_not_change_the_solution(sih):
    """options.reorder renumbers columns and rows by length on the device only;
    results come back in the caller's order and agree with the unrenumbered solve."""
    prob, entry, _ = golden_case("rand_2000x5000_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    a = sih.solve_gpu_mixed(prob, cfg, reorder=1)
    b = sih.solve_gpu_mixed(prob, cfg, reorder=0)
    assert a.is_optimal() and b.is_optimal()
    ref = entry["highs_objective"]
    for s in (a, b):
        assert abs(s.primal_objective - ref) <= 40 * 1e-6 * (1 + abs(ref))
    np.testing.assert_allclose(a.x, b.x, atol=1e-3 * max(1.0, np.abs(b.x).max()))


def test_staged_gathers_are_bit_identical(sih):
    """options.staged_kib serves gathers below the staged prefix from a
    shared-memory copy of the vector; the arithmetic is unchanged, so a solve
    with staging (forced on both SpMVs, and automatic on a Zipf LP whose prefix
    carries most nonzeros) returns the same point bit for bit."""
    from sih_pdhg.generators import zipf_lp

    prob = zipf_lp(20_000, 40_000, 480_000, seed=3)
    cfg = sih.GpuPdhgConfig(max_iterations=3000, tol_primal=1e-4, tol_dual=1e-4, tol_gap=1e-4)
    # staging belongs to the kernel-per-phase step form (persistent = 0)
    off = sih.solve_gpu_mixed(prob, cfg, staged_kib=-1, persistent=0)
    for kib in (16, 0):
        on = sih.solve_gpu_mixed(prob, cfg, staged_kib=kib, persistent=0)
        assert on.status == off.status
        assert on.simplex_iterations == off.simplex_iterations
        np.testing.assert_array_equal(on.x, off.x)
        np.testing.assert_array_equal(on.row_duals, off.row_duals)


def test_staged_kib_above_the_device_limit_is_rejected(sih):
    prob, _, _ = golden_case("rand_200x500_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=1000, tol_primal=1e-4, tol_dual=1e-4, tol_gap=1e-4)
    with pytest.raises(Exception, match="staged_kib"):
        sih.solve_gpu_mixed(prob, cfg, staged_kib=100_000)


@pytest.mark.parametrize("lanes", [(1, 1), (2, 4), (8, 2)])
def test_lane_width_override_solves(sih, lanes):
    """options.lanes_csr / lanes_csc fix the lanes per segment of the light
    SpMV tasks; any power of two gives a correct solve."""
    prob, entry, _ = golden_case("rand_2000x5000_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    s = sih.solve_gpu_mixed(prob, cfg, lanes_csr=lanes[0], lanes_csc=lanes[1])
    assert s.is_optimal()
    ref = entry["highs_objective"]
    assert abs(s.primal_objective - ref) <= 40 * 1e-6 * (1 + abs(ref))

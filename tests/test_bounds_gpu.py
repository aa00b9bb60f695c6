"""Every kind of bound on the GPU (sih_pdhg.generators.mixed_bounds_lp:
equality, <=, >=, ranged and free rows; boxed, lower-only, upper-only, free and
fixed columns; an empty row and an empty column), through the C ABI:

* mixed path: reaches 1e-6 relative KKT (rechecked on the host in FP64), stays
  inside the column bounds and matches the FP64 HiGHS objective;
* plain path in exact mode: the same bits as the plain-algorithm oracle (the
  reference's arithmetic), converged or at the iteration limit;
* a batch mixing these LPs with a random one: every instance solves as alone.
"""
import numpy as np
import pytest

from conftest import golden_case, highs_general

pytestmark = pytest.mark.gpu
SEEDS = (0, 1, 2)


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


def _lp(seed):
    from sih_pdhg.generators import mixed_bounds_lp

    return mixed_bounds_lp(seed=seed)


def _cfg(sih, tol):
    return sih.GpuPdhgConfig(max_iterations=1_000_000, tol_primal=tol, tol_dual=tol, tol_gap=tol)


@pytest.mark.parametrize("seed", SEEDS)
def test_mixed_path_solves_every_bound_kind(sih, oracle_lib, seed):
    p = _lp(seed)
    tol = 1e-6
    sol = sih.solve_gpu_mixed(p, _cfg(sih, tol))
    assert sol.status == sih.SolutionStatus.Optimal
    assert sol.rel_primal <= 2 * tol and sol.rel_dual <= 2 * tol and sol.rel_gap <= 2 * tol
    k = oracle_lib.kkt(p, sol.x, sol.row_duals)
    assert k["rel_primal"] == pytest.approx(sol.rel_primal, rel=1e-6, abs=1e-12)
    slack = 1e-6 * np.maximum(1.0, np.abs(sol.x))
    assert np.all(sol.x >= p.col_lower - slack) and np.all(sol.x <= p.col_upper + slack)
    ref, _ = highs_general(p)
    assert abs(sol.primal_objective - ref) <= 40 * tol * (1 + abs(ref))


@pytest.mark.parametrize("seed", SEEDS)
def test_exact_plain_path_is_bit_identical_to_the_oracle(sih, oracle_lib, seed):
    p = _lp(seed)
    cfg = sih.GpuPdhgConfig(max_iterations=20000)
    x_ref, y_ref, info = oracle_lib.plain_pdhg(p, cfg)
    sol = sih.GpuSolver.solve_ex(p, cfg, algorithm=sih.ALGO_PLAIN, exact_arithmetic=1)
    assert int(sol.status) == info["status"]
    assert sol.simplex_iterations == info["iterations"]
    np.testing.assert_array_equal(sol.x, x_ref)
    np.testing.assert_array_equal(sol.row_duals, y_ref)


def test_batch_with_every_bound_kind(sih):
    probs = [_lp(s) for s in SEEDS] + [golden_case("rand_200x500_k8_s0")[0]]
    tol = 1e-4
    # one launch shape for batch and single solves (no autotuning, kernels per
    # phase): each instance then computes what it computes alone
    same = dict(autotune=0, persistent=0)
    batch = sih.solve_batch(probs, _cfg(sih, tol), **same)
    for p, r in zip(probs, batch):
        single = sih.solve_gpu_mixed(p, _cfg(sih, tol), **same)
        assert r.is_optimal()
        assert r.rel_primal <= 2 * tol and r.rel_dual <= 2 * tol and r.rel_gap <= 2 * tol
        assert abs(r.simplex_iterations - single.simplex_iterations) <= 2 * 64
        ref, _ = highs_general(p)
        assert abs(r.primal_objective - ref) <= 40 * tol * (1 + abs(ref))

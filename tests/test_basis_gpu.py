"""Basis guess of the hybrid polish on the GPU (sih_pdhg_basis_guess) against
the reference's rule (oracle.basis_guess, core/src/gpu/gpu_solver.cpp:332-395):
same Basic / AtLower / AtUpper status for every column and row, including
ties in the distance (taken in candidate order) and absent bounds."""
import numpy as np
import pytest

from conftest import golden_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


def _random_case(m, n, seed):
    """A problem shell (bounds only matter) with values on a coarse grid, so
    that many distances tie, and a mix of finite, absent (+-1e20, inf) bounds."""
    from sih_pdhg.generators import small_random_lp

    rng = np.random.default_rng(seed)
    p = small_random_lp(m, n, 2, seed)
    k = n + m
    lo = rng.choice([0.0, -1.0, -np.inf, -1e20, 2.0], size=k)
    width = rng.choice([1.0, 3.0, np.inf, 1e16], size=k)
    with np.errstate(invalid="ignore"):
        hi = np.where(np.isfinite(lo), lo + width, width)  # never -inf + inf
    p.col_lower[:], p.row_lower[:] = lo[:n], lo[n:]
    p.col_upper[:], p.row_upper[:] = hi[:n], hi[n:]
    vals = np.round(rng.uniform(-2.0, 5.0, size=k) * 4.0) / 4.0  # quarter steps: ties
    return p, vals[:n], vals[n:]


@pytest.mark.parametrize("m,n,seed", [(40, 100, 0), (2000, 5000, 1), (300_000, 700_000, 2)])
def test_basis_guess_equals_reference_rule(sih, m, n, seed):
    import oracle

    p, x, ax = _random_case(m, n, seed)
    cs, rs = sih.basis_guess(p, x, ax)
    ecs, ers = oracle.basis_guess(p, x, ax)
    np.testing.assert_array_equal(cs, ecs)
    np.testing.assert_array_equal(rs, ers)
    assert int((cs == 0).sum() + (rs == 0).sum()) == m


def test_basis_guess_of_a_solved_lp(sih):
    """On a mixed-path solution (x and its FP64 row activity, the slack the
    engine returns), as GpuSolver::solve_hybrid would call it."""
    import oracle

    prob, _, _ = golden_case("rand_200x500_k8_s0")
    cfg = sih.GpuPdhgConfig(max_iterations=200000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    sol = sih.solve_gpu_mixed(prob, cfg)
    cs, rs = sih.basis_guess(prob, sol.x, sol.slack)
    ecs, ers = oracle.basis_guess(prob, sol.x, sol.slack)
    np.testing.assert_array_equal(cs, ecs)
    np.testing.assert_array_equal(rs, ers)

"""Handle and batch entry points (sih_pdhg_create/run/get_result/destroy,
sih_pdhg_solve_batch, sih_pdhg_time_kernels) through the C ABI."""
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


def cfg(sih, tol=1e-4):
    return sih.GpuPdhgConfig(max_iterations=200000, tol_primal=tol, tol_dual=tol, tol_gap=tol)


def test_handle_runs_are_deterministic(sih):
    """Every reduction has a fixed order, so two runs give the same bits."""
    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        h.run()
        a = h.result(0)
        h.run()
        b = h.result(0)
    assert a.is_optimal() and a.simplex_iterations == b.simplex_iterations
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.row_duals, b.row_duals)


def test_handle_matches_one_shot_solve(sih):
    prob, _, _ = golden_case("rand_200x500_k8_s0")
    one = sih.solve_gpu_mixed(prob, cfg(sih))
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        h.run()
        r = h.result(0)
    assert r.simplex_iterations == one.simplex_iterations
    np.testing.assert_array_equal(r.x, one.x)


def test_batch_matches_single_solves(sih):
    """Instances of a batch reach their own tolerance and objective; the batch
    shares kernels, not state, so each follows (nearly) its single-solve path."""
    names = ["rand_50x120_k4_s1", "rand_200x500_k8_s0", "rand_2000x5000_k8_s0", "toy04_lp_equality_ranges",
             "rand_100x250_k6_s0"]
    probs = [golden_case(n)[0] for n in names]
    entries = [golden_case(n)[1] for n in names]
    # one launch shape for batch and single solves (no autotuning, kernels per
    # phase): each instance then computes what it computes alone
    same = dict(autotune=0, persistent=0)
    batch = sih.solve_batch(probs, cfg(sih), **same)
    for p, e, r in zip(probs, entries, batch):
        single = sih.solve_gpu_mixed(p, cfg(sih), **same)
        assert r.is_optimal()
        assert r.rel_primal <= 2e-4 and r.rel_gap <= 2e-4
        assert abs(r.simplex_iterations - single.simplex_iterations) <= 2 * 64
        ref = e["highs_objective"]
        assert abs(r.primal_objective - ref) <= 4e-3 * (1 + abs(ref))


def test_batch_of_identical_instances_is_identical(sih):
    prob, _, _ = golden_case("rand_200x500_k8_s0")
    batch = sih.solve_batch([prob, prob, prob], cfg(sih))
    for r in batch[1:]:
        assert r.simplex_iterations == batch[0].simplex_iterations
        np.testing.assert_allclose(r.x, batch[0].x, rtol=0, atol=1e-5)


def test_plain_batch_is_sequential_reference_solves(sih):
    probs = [golden_case(n)[0] for n in ("rand_50x120_k4_s1", "toy01_lp_simple")]
    c = sih.GpuPdhgConfig(max_iterations=6000)
    batch = sih.solve_batch(probs, c, algorithm=sih.ALGO_PLAIN)
    for p, r in zip(probs, batch):
        single = sih.solve_gpu_pdhg(p, c)
        assert r.simplex_iterations == single.simplex_iterations
        np.testing.assert_array_equal(r.x, single.x)


def test_time_kernels(sih):
    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        secs, byts = h.time_kernels(5)
        h.run()
        assert h.result(0).is_optimal()
    assert all(s > 0 for s in secs) and all(b > 0 for b in byts)


def test_result_before_run_is_an_error(sih):
    prob, _, _ = golden_case("toy01_lp_simple")
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        with pytest.raises(sih.SihPdhgError):
            h.result(0)
        with pytest.raises(sih.SihPdhgError):
            h.result(3)


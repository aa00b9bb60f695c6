"""Persistent step kernel (options.persistent): one cooperative launch per
evaluation period runs the period's steps as phases separated by grid
barriers.  It must give the same iterates as the kernel-per-phase CUDA-graph
path (same tasks, reduction order and controller), and its barrier's bounded
wait must end a kernel whose blocks stop arriving without hanging the GPU."""
import ctypes as C

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


@pytest.mark.parametrize("name", ["rand_200x500_k8_s0", "rand_2000x5000_k8_s0", "toy04_lp_equality_ranges"])
def test_persistent_equals_graph_path(sih, name):
    prob, _, _ = golden_case(name)
    a = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), persistent=0)
    b = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), persistent=1)
    assert a.is_optimal() and b.is_optimal()
    assert a.simplex_iterations == b.simplex_iterations and a.restarts == b.restarts
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.row_duals, b.row_duals)


def test_persistent_batch_equals_graph_batch(sih):
    """A batch whose instances stop at different evaluations: the compaction
    between persistent launches drops finished instances as in the graph path."""
    from sih_pdhg.generators import mixed_bounds_lp, refinery_lp, small_random_lp

    probs = [small_random_lp(300, 700, 6, 3), mixed_bounds_lp(seed=1), refinery_lp(24, 1), small_random_lp(50, 120, 4, 2)]
    a = sih.solve_batch(probs, cfg(sih), persistent=0)
    b = sih.solve_batch(probs, cfg(sih), persistent=1)
    iters = {r.simplex_iterations for r in a}
    assert len(iters) > 1, "instances should stop at different evaluations"
    for ra, rb in zip(a, b):
        assert ra.status == rb.status and ra.simplex_iterations == rb.simplex_iterations
        np.testing.assert_array_equal(ra.x, rb.x)
        np.testing.assert_array_equal(ra.row_duals, rb.row_duals)


def test_persistent_handle_reruns_are_identical(sih):
    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED, persistent=1) as h:
        h.run()
        a = h.result(0)
        h.run()
        b = h.result(0)
    assert a.is_optimal() and a.simplex_iterations == b.simplex_iterations
    np.testing.assert_array_equal(a.x, b.x)


def _barrier(sih, blocks, missing, rounds, limit):
    lib = sih._lib.load()
    t, p = C.c_int32(-1), C.c_int32(-1)
    sih._lib.check(lib.sih_pdhg_check_grid_barrier(blocks, missing, rounds, limit, C.byref(t), C.byref(p)))
    return t.value, p.value


def test_grid_barrier_completes_every_round(sih):
    assert _barrier(sih, 152, 0, 50, 1.0) == (0, 50)


def test_grid_barrier_wait_runs_out_and_the_device_stays_usable(sih):
    """A barrier that waits for one block more than the grid holds (an
    arrival nothing makes): every block's bounded wait runs out after the
    limit, the kernel returns and the status says so; the context still solves."""
    import time

    t0 = time.perf_counter()
    timed_out, passed = _barrier(sih, 8, 1, 3, 0.05)
    assert timed_out == 1 and passed == 0
    assert time.perf_counter() - t0 < 5.0
    prob, _, _ = golden_case("rand_200x500_k8_s0")
    assert sih.solve_gpu_mixed(prob, cfg(sih), persistent=1).is_optimal()


@pytest.mark.parametrize("name", ["rand_200x500_k8_s0", "rand_2000x5000_k8_s0", "toy04_lp_equality_ranges"])
def test_single_lp_persistent_form_solves_like_the_graph_path(sih, name):
    """options.persistent = 2: static task shares and per-block partials give
    other roundings than the ticket chain, so the trajectory may differ in the
    last bits: same status, tolerance reached, the same optimum."""
    prob, entry, _ = golden_case(name)
    a = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), persistent=0)
    b = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), persistent=2)
    assert a.is_optimal() and b.is_optimal()
    assert max(b.rel_primal, b.rel_dual, b.rel_gap) <= 2e-6
    assert abs(b.simplex_iterations - a.simplex_iterations) <= max(4 * 64, 0.2 * a.simplex_iterations)
    ref = entry["highs_objective"]
    assert abs(b.primal_objective - ref) <= 4e-6 * (1 + abs(ref))


def test_single_lp_persistent_form_is_deterministic(sih):
    from sih_pdhg.generators import refinery_lp

    prob = refinery_lp(24, 2)
    with sih.PdhgHandle(prob, cfg(sih), algorithm=sih.ALGO_MIXED, persistent=2) as h:
        h.run()
        a = h.result(0)
        h.run()
        b = h.result(0)
    assert a.is_optimal() and a.simplex_iterations == b.simplex_iterations
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.row_duals, b.row_duals)


def test_automatic_form_and_launch_shape(sih):
    """persistent = -1 (default): the single-LP form for a small LP, kernels per
    phase for a large one; a batch is autotuned (autotune = -1) and reports the
    shape it chose; a second handle of the same shape reuses it."""
    from sih_pdhg.generators import small_random_lp

    small = small_random_lp(200, 500, 8, 0)
    with sih.PdhgHandle(small, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        sh = h.launch_shape()
        assert sh["persistent"] == 2 and sh["tuned"] == 0
    batch = [small_random_lp(300, 700, 6, s) for s in range(3)]
    with sih.PdhgHandle(batch, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        sh = h.launch_shape()
        h.run()
        res = [h.result(b) for b in range(3)]
    assert sh["tuned"] == 1 and sh["persistent"] in (0, 1)
    assert sh["row_lanes"] in (0, 1, 2, 4, 8) and sh["col_lanes"] in (0, 1, 2, 4, 8)
    assert all(r.is_optimal() for r in res)
    with sih.PdhgHandle(batch, cfg(sih), algorithm=sih.ALGO_MIXED) as h:
        assert h.launch_shape() == sh


def test_packed_steps_equal_three_kernel_steps(sih):
    """options.packed: two kernels per step (the elementwise primal step folded
    into the SpMVs, x' computed from packed column records) give the iterates
    of the three-kernel step bit for bit, on a single LP and on a batch whose
    instances restart and stop at different evaluations."""
    from sih_pdhg.generators import mixed_bounds_lp, refinery_lp, small_random_lp

    prob, _, _ = golden_case("rand_2000x5000_k8_s0")
    kw = dict(persistent=0, autotune=0, staged_kib=-1)
    a = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), packed=0, **kw)
    b = sih.solve_gpu_mixed(prob, cfg(sih, 1e-6), packed=1, **kw)
    assert a.is_optimal() and a.simplex_iterations == b.simplex_iterations and a.restarts == b.restarts
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.row_duals, b.row_duals)
    probs = [small_random_lp(300, 700, 6, 3), mixed_bounds_lp(seed=1), refinery_lp(24, 1), small_random_lp(50, 120, 4, 2)]
    ra = sih.solve_batch(probs, cfg(sih), packed=0, **kw)
    rb = sih.solve_batch(probs, cfg(sih), packed=1, **kw)
    for x, y in zip(ra, rb):
        assert x.status == y.status and x.simplex_iterations == y.simplex_iterations
        np.testing.assert_array_equal(x.x, y.x)
        np.testing.assert_array_equal(x.row_duals, y.row_duals)
    with sih.PdhgHandle(probs, cfg(sih), algorithm=sih.ALGO_MIXED, packed=1, **kw) as h:
        sh = h.launch_shape()
        secs, byts = h.time_kernels(3)
    assert sh["packed"] == 1 and secs[0] == 0.0 and secs[1] > 0 and secs[2] > 0

"""Gradients of the optimal value of the differentiable-layer LPs (the
envelope theorem: d obj / d b = the optimal duals), on the GPU.

* small LPs through the torch layer (lp_layer(..., return_objective=True)):
  d obj / d bounds against the FP64 HiGHS duals of the golden cases;
* four LPs of the layer's size (layer_lp(seed), 20,000 x 50,000, 10 nonzeros
  per column) solved as one batch to 1e-6: d obj / d b from the returned point
  against FP64 duals of the oracle at relative KKT 1e-9 (the fixture
  tests/golden/layer_duals.npz, written by tests/golden/make_layer_duals.py),
  relative error <= 1e-3."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


def test_layer_objective_gradient_is_the_simplex_dual(sih):
    torch = pytest.importorskip("torch")
    from sih_pdhg.layer import lp_layer

    names = ["rand_100x250_k6_s0", "rand_200x500_k8_s0"]
    cases = [golden_case(n) for n in names]
    probs = [c[0] for c in cases]
    # same shapes are required per call: one call per case
    for (p, entry, vec), name in zip(cases, names):
        t = lambda a: torch.tensor(np.asarray(a)[None, :], dtype=torch.float64, requires_grad=True)
        c, rl, ru, l, u = (t(p.c), t(p.row_lower), t(p.row_upper), t(p.col_lower), t(p.col_upper))
        x, v = lp_layer([p.A], c, rl, ru, l, u, return_objective=True)
        ref = entry["highs_objective"]
        assert float(v[0].detach()) == pytest.approx(ref, rel=1e-5)
        v.sum().backward()
        db = (rl.grad + ru.grad).numpy()[0]
        y_highs = vec["highs/row_duals"] if "highs/row_duals" in vec.files else None
        if y_highs is not None:
            scale = max(1.0, np.abs(y_highs).max())
            assert np.abs(db - y_highs).max() <= 1e-4 * scale, name
        np.testing.assert_allclose(c.grad.numpy()[0], x.detach().numpy()[0])


def test_layer_size_objective_gradient_matches_fp64_duals(sih):
    """The done-bar of the layer at its size: on 4 of the 64 layer LPs, d obj / d b
    from the GPU solution agrees with the FP64 duals to 1e-3 relative error."""
    from sih_pdhg.generators import layer_lp
    from sih_pdhg.layer import objective_gradients

    path = os.path.join(GOLDEN, "layer_duals.npz")
    ref = np.load(path)
    seeds = [0, 1, 2, 3]
    probs = [layer_lp(s) for s in seeds]
    cfg = sih.GpuPdhgConfig(max_iterations=1_000_000, tol_primal=1e-6, tol_dual=1e-6, tol_gap=1e-6)
    sols = sih.solve_batch(probs, cfg)
    for s, p, sol in zip(seeds, probs, sols):
        assert sol.is_optimal()
        g = objective_gradients(p, sol.x, sol.row_duals)
        db = g["row_lower"] + g["row_upper"]
        y = ref[f"y{s}"].astype(np.float64)
        err = np.linalg.norm(db - y) / np.linalg.norm(y)
        print(f"seed {s}: {sol.simplex_iterations} steps, |d obj/d b - y*| / |y*| = {err:.2e}, "
              f"objective {g['objective']:.10g} vs {float(ref[f'obj{s}']):.10g}")
        assert err <= 1e-3
        assert g["objective"] == pytest.approx(float(ref[f"obj{s}"]), rel=2e-6)


def test_layer_size_value_gradients_through_torch_without_polish(sih):
    """The torch layer at the layer's size, polish off: one batched solve
    forward, the optimal values' gradients (duals) backward; d v / d b against
    the FP64 duals of the fixture."""
    torch = pytest.importorskip("torch")
    from sih_pdhg.generators import layer_lp
    from sih_pdhg.layer import lp_layer

    ref = np.load(os.path.join(GOLDEN, "layer_duals.npz"))
    probs = [layer_lp(s) for s in (0, 1)]
    st = lambda k: torch.tensor(np.stack([getattr(p, k) for p in probs]), dtype=torch.float64, requires_grad=True)
    c, rl, ru, l, u = st("c"), st("row_lower"), st("row_upper"), st("col_lower"), st("col_upper")
    x, v = lp_layer([p.A for p in probs], c, rl, ru, l, u, return_objective=True, polish=False)
    v.sum().backward()
    db = (rl.grad + ru.grad).numpy()
    for k in range(2):
        y = ref[f"y{k}"].astype(np.float64)
        assert np.linalg.norm(db[k] - y) / np.linalg.norm(y) <= 1e-3
        assert float(v[k].detach()) == pytest.approx(float(ref[f"obj{k}"]), rel=2e-6)
    np.testing.assert_allclose(c.grad.numpy(), x.detach().numpy())

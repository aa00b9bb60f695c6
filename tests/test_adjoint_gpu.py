"""Basis polish (sih_pdhg_polish_batch), adjoint of the LP solution map
(sih_pdhg_adjoint_batch) and the torch autograd layer (sih_pdhg.layer):
the polished vertex and duals against FP64 HiGHS, gradients of the objective
against the simplex duals (d obj / d b = y*, HiGHS marginals) and gradients of
L = |x* - t|^2 + 0.1 c^T x* against central finite differences of FP64 HiGHS
re-solves (h = 1e-4), to 1e-3 relative error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-4


@pytest.fixture(scope="module")
def sih():
    import sih_pdhg

    if not sih_pdhg.GpuSolver.is_cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    return sih_pdhg


def _highs(p, c=None, rl=None, ru=None, u=None):
    sp = pytest.importorskip("scipy.sparse")
    from scipy.optimize import linprog

    c = p.c if c is None else c
    rl = p.row_lower if rl is None else rl
    ru = p.row_upper if ru is None else ru
    u = p.col_upper if u is None else u
    A = sp.csc_matrix((p.A.csc_values(), p.A.csc_row_ind(), p.A.csc_col_ptr()), shape=(p.num_rows(), p.num_cols()))
    eq = rl == ru
    ub = (~eq) & (ru < 1e20)
    lb = (~eq) & (rl > -1e20)
    r = linprog(c, A_ub=sp.vstack([A[ub], -A[lb]]).tocsc(), b_ub=np.concatenate([ru[ub], -rl[lb]]), A_eq=A[eq],
                b_eq=rl[eq], bounds=list(zip(p.col_lower, u)), method="highs-ds")
    assert r.status == 0
    y = np.zeros(p.num_rows())
    y[eq] = r.eqlin.marginals
    y[ub] += r.ineqlin.marginals[: ub.sum()]
    y[lb] -= r.ineqlin.marginals[ub.sum():]
    return r.x, y


def _solve(sih, p, tol=1e-6):
    cfg = sih.GpuPdhgConfig(max_iterations=1_000_000, tol_primal=tol, tol_dual=tol, tol_gap=tol)
    s = sih.solve_gpu_mixed(p, cfg)
    assert s.is_optimal()
    return s


@pytest.mark.parametrize("shape", [(50, 120, 4, 1), (100, 250, 6, 0), (200, 500, 8, 0)])
def test_objective_gradient_is_the_simplex_duals(sih, shape):
    from sih_pdhg.generators import small_random_lp

    m, n, k, seed = shape
    p = small_random_lp(m, n, k, seed)
    s = _solve(sih, p)
    _, y = _highs(p)
    grads, info = sih.adjoint_batch([p], [s.x], [s.row_duals], [p.c], tolerance=1e-7)
    gb = grads[0]["row_lower"] + grads[0]["row_upper"]
    assert info[0]["status"] == 0 and info[0]["free_columns"] == info[0]["active_rows"]
    assert np.linalg.norm(gb - y) <= 1e-3 * np.linalg.norm(y)
    assert not np.any(grads[0]["c"])  # x* does not move with c


@pytest.mark.parametrize("shape", [(50, 120, 4, 1), (100, 250, 6, 0), (200, 500, 8, 0)])
def test_polish_recovers_the_optimal_vertex(sih, shape):
    from sih_pdhg.generators import small_random_lp

    m, n, k, seed = shape
    p = small_random_lp(m, n, k, seed)
    s = _solve(sih, p)
    xs, ys, infos = sih.polish_batch([p], [s.x], [s.row_duals])
    info = infos[0]
    x_ref, y_ref = _highs(p)
    assert info["status"] == 0 and info["free_columns"] == info["active_rows"]
    assert info["primal_residual"] <= 1e-9 and info["dual_residual"] <= 1e-9
    # an optimal basis: no bound or sign violation beyond rounding
    assert info["primal_violation"] <= 1e-9 and info["dual_violation"] <= 1e-9
    assert np.abs(xs[0] - x_ref).max() <= 1e-7 * max(1.0, np.abs(x_ref).max())
    assert np.abs(-ys[0] - y_ref).max() <= 1e-7 * max(1.0, np.abs(y_ref).max())
    # the PDHG point itself is only 1e-6 accurate
    assert abs(p.c @ xs[0] - p.c @ x_ref) <= 1e-9 * abs(p.c @ x_ref)


def test_polish_flags_a_basis_that_is_not_optimal(sih):
    """On 2000 x 5000 the basis read off the FP32 PDHG point at 1e-6 misses a
    few near-degenerate columns; the polish must then say so through its
    violation fields rather than return a wrong vertex silently."""
    from sih_pdhg.generators import small_random_lp

    p = small_random_lp(2000, 5000, 8, 0)
    s = _solve(sih, p)
    xs, _, infos = sih.polish_batch([p], [s.x], [s.row_duals])
    info = infos[0]
    x_ref, _ = _highs(p)
    exact = np.abs(xs[0] - x_ref).max() <= 1e-7 * max(1.0, np.abs(x_ref).max())
    flagged = info["primal_violation"] > 1e-9 or info["dual_violation"] > 1e-9
    assert info["free_columns"] == info["active_rows"]
    assert exact or flagged


@pytest.mark.parametrize("shape", [(100, 250, 6, 0), (200, 500, 8, 0)])
def test_loss_gradient_matches_finite_differences(sih, shape):
    """At the polished vertex (the layer's output) the adjoint gradient is the
    derivative that FP64 re-solves measure."""
    from sih_pdhg.generators import small_random_lp

    m, n, k, seed = shape
    p = small_random_lp(m, n, k, seed)
    s = _solve(sih, p)
    xs, ys, _ = sih.polish_batch([p], [s.x], [s.row_duals])
    rng = np.random.default_rng(3)
    xt = rng.uniform(0, p.col_upper)
    g = 2 * (xs[0] - xt) + 0.1 * p.c
    grads, _ = sih.adjoint_batch([p], [xs[0]], [ys[0]], [g], tolerance=1e-7)
    G = grads[0]

    def loss(c=None, rl=None, ru=None, u=None):
        x, _ = _highs(p, c=c, rl=rl, ru=ru, u=u)
        cc = p.c if c is None else c
        return np.sum((x - xt) ** 2) + 0.1 * cc @ x

    fin_l, fin_u = p.row_lower > -1e20, p.row_upper < 1e20
    for _ in range(2):
        db = rng.standard_normal(m)
        fd = (loss(rl=p.row_lower + H * db * fin_l, ru=p.row_upper + H * db * fin_u)
              - loss(rl=p.row_lower - H * db * fin_l, ru=p.row_upper - H * db * fin_u)) / (2 * H)
        ad = (G["row_lower"] * fin_l + G["row_upper"] * fin_u) @ db
        assert abs(ad - fd) <= 1e-3 * abs(fd)
        du = rng.standard_normal(n)
        fd = (loss(u=p.col_upper + H * du) - loss(u=p.col_upper - H * du)) / (2 * H)
        assert abs(G["col_upper"] @ du - fd) <= 1e-3 * abs(fd)
        dc = rng.standard_normal(n)
        fd = (loss(c=p.c + H * dc) - loss(c=p.c - H * dc)) / (2 * H)
        assert abs(0.1 * xs[0] @ dc - fd) <= 1e-3 * abs(fd)  # explicit part only


def test_torch_layer_backward_equals_adjoint(sih):
    torch = pytest.importorskip("torch")
    from sih_pdhg.generators import small_random_lp
    from sih_pdhg.layer import lp_layer

    probs = [small_random_lp(100, 250, 6, s) for s in range(3)]
    mats = [p.A for p in probs]
    t64 = lambda key: torch.tensor(np.stack([getattr(p, key) for p in probs]), dtype=torch.float64,
                                   requires_grad=True)
    c, rl, ru, l, u = (t64(k) for k in ("c", "row_lower", "row_upper", "col_lower", "col_upper"))
    x = lp_layer(mats, c, rl, ru, l, u)
    target = torch.zeros_like(x)
    loss = ((x - target) ** 2).sum() + 0.1 * (c * x).sum()
    loss.backward()
    # the layer returns the optimal vertex; its gradients are the adjoint's there
    for i, p in enumerate(probs):
        x_ref, _ = _highs(p)
        xi = x[i].detach().numpy()
        assert np.abs(xi - x_ref).max() <= 1e-7 * max(1.0, np.abs(x_ref).max())
        g = 2 * xi + 0.1 * p.c
        _, y_ref = _highs(p)
        grads, _ = sih.adjoint_batch([p], [xi], [-y_ref], [g], tolerance=1e-7)
        rel = lambda a, b: np.linalg.norm(a - b) / max(1e-12, np.linalg.norm(b))
        assert rel(rl.grad[i].numpy(), grads[0]["row_lower"]) <= 1e-6
        assert rel(u.grad[i].numpy(), grads[0]["col_upper"]) <= 1e-6
        assert rel(c.grad[i].numpy(), 0.1 * xi) <= 1e-12

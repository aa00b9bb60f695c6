"""The reference-compatible launchers (include/sih_pdhg.h sih_pdhg_launch_*)
against the oracle's restatement of core/src/gpu/cuda_pdhg.cu kernels.
SpMVs: FP32 tolerance (different summation order); elementwise kernels:
bit for bit (same unfused float operations)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import oracle
    import sih_pdhg
    from sih_pdhg import _lib

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch, _lib.load(), oracle


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("shape", [(2000, 5000, 8), (300, 700, 40), (50, 60, 1)])
def test_spmv_launchers(env, shape):
    torch, lib, oracle = env
    from sih_pdhg.generators import small_random_lp

    m, n, k = shape
    p = small_random_lp(m, n, k, 4)
    A = p.A
    rp, ci, rv = A.csr_row_ptr().astype(np.int32), A.csr_col_ind().astype(np.int32), A.csr_values().astype(np.float32)
    cp, ri, cv = A.csc_col_ptr().astype(np.int32), A.csc_row_ind().astype(np.int32), A.csc_values().astype(np.float32)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(m).astype(np.float32)
    d = {k2: _dev(torch, v) for k2, v in dict(rp=rp, ci=ci, rv=rv, cp=cp, ri=ri, cv=cv, x=x, y=y).items()}
    ax = torch.zeros(m, dtype=torch.float32, device="cuda")
    aty = torch.zeros(n, dtype=torch.float32, device="cuda")
    assert lib.sih_pdhg_launch_csr_spmv(m, d["rp"].data_ptr(), d["ci"].data_ptr(), d["rv"].data_ptr(),
                                        d["x"].data_ptr(), ax.data_ptr(), None) == 0
    assert lib.sih_pdhg_launch_csc_spmv(n, d["cp"].data_ptr(), d["ri"].data_ptr(), d["cv"].data_ptr(),
                                        d["y"].data_ptr(), aty.data_ptr(), None) == 0
    torch.cuda.synchronize()
    ref_ax = oracle.csr_spmv_f32(rp, ci, rv, x)
    ref_aty = oracle.csc_spmv_f32(cp, ri, cv, y)
    # FP32 sums of k terms: |error| <= k * eps * sum |a_i x_i|
    abs_ax = np.bincount(np.repeat(np.arange(m), np.diff(rp)), weights=np.abs(rv * x[ci]), minlength=m)
    abs_aty = np.bincount(np.repeat(np.arange(n), np.diff(cp)), weights=np.abs(cv * y[ri]), minlength=n)
    tol_ax = 2 * max(1, np.diff(rp).max()) * 1.2e-7 * abs_ax + 1e-30
    tol_aty = 2 * max(1, np.diff(cp).max()) * 1.2e-7 * abs_aty + 1e-30
    assert np.all(np.abs(ax.cpu().numpy() - ref_ax) <= tol_ax)
    assert np.all(np.abs(aty.cpu().numpy() - ref_aty) <= tol_aty)


def test_update_launchers_bit_exact(env):
    torch, lib, oracle = env
    rng = np.random.default_rng(2)
    n, m = 10_001, 7_003
    tau = rng.uniform(0.01, 1, n).astype(np.float32)
    c = rng.standard_normal(n).astype(np.float32)
    aty = rng.standard_normal(n).astype(np.float32)
    l = np.where(rng.random(n) < 0.1, -np.inf, rng.uniform(-1, 0, n)).astype(np.float32)
    u = np.where(rng.random(n) < 0.1, np.inf, rng.uniform(0, 2, n)).astype(np.float32)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    sig = rng.uniform(0.01, 1, m).astype(np.float32)
    axb = rng.standard_normal(m).astype(np.float32)
    rl = np.where(rng.random(m) < 0.5, -np.inf, rng.uniform(-1, 0, m)).astype(np.float32)
    ru = np.where(rng.random(m) < 0.3, np.inf, rng.uniform(0, 1, m)).astype(np.float32)
    ru[:100] = rl[:100] = 0.25  # equality rows
    y = rng.standard_normal(m).astype(np.float32)
    d = {k: _dev(torch, v) for k, v in dict(tau=tau, c=c, aty=aty, l=l, u=u, x=x, sig=sig, axb=axb, rl=rl, ru=ru,
                                               y=y).items()}
    xbar = torch.zeros(n, dtype=torch.float32, device="cuda")
    assert lib.sih_pdhg_launch_primal_update(n, d["tau"].data_ptr(), d["c"].data_ptr(), d["aty"].data_ptr(),
                                             d["l"].data_ptr(), d["u"].data_ptr(), d["x"].data_ptr(),
                                             xbar.data_ptr(), None) == 0
    assert lib.sih_pdhg_launch_dual_update(m, d["sig"].data_ptr(), d["axb"].data_ptr(), d["rl"].data_ptr(),
                                           d["ru"].data_ptr(), d["y"].data_ptr(), None) == 0
    rv = torch.zeros(m, dtype=torch.float32, device="cuda")
    cvl = torch.zeros(n, dtype=torch.float32, device="cuda")
    assert lib.sih_pdhg_launch_residuals(m, n, d["axb"].data_ptr(), d["rl"].data_ptr(), d["ru"].data_ptr(),
                                         rv.data_ptr(), d["x"].data_ptr(), d["c"].data_ptr(), d["aty"].data_ptr(),
                                         d["l"].data_ptr(), d["u"].data_ptr(), d["tau"].data_ptr(),
                                         cvl.data_ptr(), None) == 0
    xb2 = torch.zeros(n, dtype=torch.float32, device="cuda")
    assert lib.sih_pdhg_launch_restart(n, d["x"].data_ptr(), xb2.data_ptr(), None) == 0
    torch.cuda.synchronize()
    x_ref, xbar_ref = oracle.primal_update_f32(tau, c, aty, l, u, x)
    y_ref = oracle.dual_update_f32(sig, axb, rl, ru, y)
    np.testing.assert_array_equal(d["x"].cpu().numpy(), x_ref)
    np.testing.assert_array_equal(xbar.cpu().numpy(), xbar_ref)
    np.testing.assert_array_equal(d["y"].cpu().numpy(), y_ref)
    np.testing.assert_array_equal(xb2.cpu().numpy(), x_ref)
    # residual maps (cuda_pdhg.cu:114-151) recomputed in numpy float32
    a = axb
    viol = np.zeros(m, np.float32)
    lo = (rl > -1e15) & (a < rl)
    viol[lo] = (rl - a)[lo]
    hi = (ru < 1e15) & (a > ru)
    viol[hi] = np.maximum(viol[hi], (a - ru)[hi])
    np.testing.assert_array_equal(rv.cpu().numpy(), viol)
    xn = x_ref
    proj = (xn - tau * (c + aty)).astype(np.float32)
    proj = np.minimum(np.maximum(proj, l), u)
    meas = (np.abs(xn - proj) / np.maximum(np.float32(1e-4), tau)).astype(np.float32)
    np.testing.assert_array_equal(cvl.cpu().numpy(), meas)

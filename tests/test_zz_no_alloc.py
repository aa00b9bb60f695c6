"""The allocation-free convergence check (sih_pdhg_check_norms_noalloc).

Callers that cannot allocate device memory while they run (a fixed device
pool handed out at start-up, or a loop where the synchronising cudaMalloc /
cudaFree are not allowed) hold every input and output themselves; the check's
working arrays live in a file-scope device array of the library.  Its two
outputs must equal what the allocating route gives: the reference launchers
sih_pdhg_launch_csr_spmv / _csc_spmv / _residuals into caller buffers,
followed by the reference's host maximum (gpu_solver.cpp:249-259).  Two calls
in a row on different problems check that the shared array's old contents do
not leak into a result.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import sih_pdhg
    from sih_pdhg import _lib

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch, _lib.load(), sih_pdhg


def _device_problem(torch, seed, m, n, k, nan_cost_column=None):
    from sih_pdhg.generators import small_random_lp

    p = small_random_lp(m, n, k, seed)
    A = p.A
    rng = np.random.default_rng(seed + 100)
    host = dict(rp=A.csr_row_ptr().astype(np.int32), ci=A.csr_col_ind().astype(np.int32),
                rv=A.csr_values().astype(np.float32), cp=A.csc_col_ptr().astype(np.int32),
                ri=A.csc_row_ind().astype(np.int32), cv=A.csc_values().astype(np.float32),
                x=rng.uniform(-1, 12, n).astype(np.float32), y=rng.standard_normal(m).astype(np.float32),
                c=p.c.astype(np.float32), l=p.col_lower.astype(np.float32), u=p.col_upper.astype(np.float32),
                tau=rng.uniform(0.01, 0.5, n).astype(np.float32), rl=p.row_lower.astype(np.float32),
                ru=p.row_upper.astype(np.float32))
    if nan_cost_column is not None:  # that column's measure is NaN; the row side is untouched
        host["c"][nan_cost_column] = np.nan
    dev = {k2: torch.from_numpy(v).cuda() for k2, v in host.items()}
    max_b = np.float32(max(1.0, np.abs(np.concatenate([host["ru"][host["ru"] < 1e15],
                                                        host["rl"][host["rl"] > -1e15]])).max()))
    max_c = np.float32(max(1.0, np.nanmax(np.abs(host["c"]))))
    return p, dev, max_b, max_c


def _allocating_route(torch, lib, p, d, max_b, max_c):
    m, n = p.num_rows(), p.num_cols()
    f = lambda k: torch.zeros(k, dtype=torch.float32, device="cuda")
    ax, aty, rv, cvl = f(m), f(n), f(m), f(n)
    assert lib.sih_pdhg_launch_csr_spmv(m, d["rp"].data_ptr(), d["ci"].data_ptr(), d["rv"].data_ptr(),
                                        d["x"].data_ptr(), ax.data_ptr(), None) == 0
    assert lib.sih_pdhg_launch_csc_spmv(n, d["cp"].data_ptr(), d["ri"].data_ptr(), d["cv"].data_ptr(),
                                        d["y"].data_ptr(), aty.data_ptr(), None) == 0
    assert lib.sih_pdhg_launch_residuals(m, n, ax.data_ptr(), d["rl"].data_ptr(), d["ru"].data_ptr(), rv.data_ptr(),
                                         d["x"].data_ptr(), d["c"].data_ptr(), aty.data_ptr(), d["l"].data_ptr(),
                                         d["u"].data_ptr(), d["tau"].data_ptr(), cvl.data_ptr(), None) == 0
    torch.cuda.synchronize()
    rows, cols = rv.cpu().numpy(), cvl.cpu().numpy()
    # the reference's host maximum keeps the running value on a NaN measure
    max_p = np.float32(max([0.0] + [v for v in rows if v == v]))
    max_d = np.float32(max([0.0] + [v for v in cols if v == v]))
    return np.float32(max_p / max_b), np.float32(max_d / max_c)


def _no_alloc_route(torch, lib, p, d, max_b, max_c, out=None):
    if out is None:
        out = torch.full((2,), -1.0, dtype=torch.float32, device="cuda")
    rc = lib.sih_pdhg_check_norms_noalloc(
        p.num_rows(), p.num_cols(), p.num_nonzeros(), d["rp"].data_ptr(), d["ci"].data_ptr(), d["rv"].data_ptr(),
        d["cp"].data_ptr(), d["ri"].data_ptr(), d["cv"].data_ptr(), d["x"].data_ptr(), d["y"].data_ptr(),
        d["c"].data_ptr(), d["l"].data_ptr(), d["u"].data_ptr(), d["tau"].data_ptr(), d["rl"].data_ptr(),
        d["ru"].data_ptr(), C.c_float(float(max_b)), C.c_float(float(max_c)), out.data_ptr(), None)
    assert rc == 0, lib.sih_pdhg_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_no_alloc_matches_allocating_route_twice(env):
    torch, lib, _ = env
    # a larger problem first, then a smaller one: stale entries of the first
    # call sit past the second call's rows and columns and must not count
    for seed, m, n, k in ((11, 3000, 9000, 12), (12, 400, 900, 6)):
        p, d, max_b, max_c = _device_problem(torch, seed, m, n, k)
        ref = _allocating_route(torch, lib, p, d, max_b, max_c)
        got = _no_alloc_route(torch, lib, p, d, max_b, max_c)
        np.testing.assert_allclose(got, np.array(ref, dtype=np.float32), rtol=1e-6, atol=0)
        assert got[0] > 0 and got[1] > 0


def test_no_alloc_rejects_sizes_beyond_its_limit(env):
    _, lib, sih = env
    rc = lib.sih_pdhg_check_norms_noalloc(400000, 200000, 10, *([None] * 14), C.c_float(1.0), C.c_float(1.0),
                                          None, None)
    assert rc == 1
    assert b"no-alloc limit" in lib.sih_pdhg_last_error()


def test_no_alloc_skips_a_nan_column_measure(env):
    """A NaN in one column's cost makes that column's measure NaN; the reference's
    host loop (gpu_solver.cpp:249-259) keeps its running maximum on a NaN, and so
    does the no-alloc check: both routes give the same finite maxima."""
    torch, lib, _ = env
    p, d, max_b, max_c = _device_problem(torch, 21, 500, 1200, 8, nan_cost_column=37)
    ref = _allocating_route(torch, lib, p, d, max_b, max_c)
    got = _no_alloc_route(torch, lib, p, d, max_b, max_c)
    assert np.all(np.isfinite(got)) and got[1] > 0
    np.testing.assert_allclose(got, np.array(ref, dtype=np.float32), rtol=1e-6, atol=0)


def test_no_alloc_calls_leave_device_memory_unchanged(env):
    """After the first call on the device (which may make CUDA load the library's
    device code and place the array), further calls allocate nothing: the
    device's free memory reads the same before and after them."""
    torch, lib, _ = env
    p, d, max_b, max_c = _device_problem(torch, 31, 800, 2000, 8)
    out = torch.full((2,), -1.0, dtype=torch.float32, device="cuda")
    first = _no_alloc_route(torch, lib, p, d, max_b, max_c, out)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        got = _no_alloc_route(torch, lib, p, d, max_b, max_c, out)
        np.testing.assert_array_equal(got, first)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)

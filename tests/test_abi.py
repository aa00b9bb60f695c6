"""The C ABI library loads, exports every declared symbol, and its structs
have the layout the Python binding (and the reference's config struct) use."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO

HEADER_DIR = os.path.join(REPO, "include")


def declared_functions():
    names = []
    for h in sorted(os.listdir(HEADER_DIR)):
        if h.endswith(".h"):
            text = open(os.path.join(HEADER_DIR, h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sih_pdhg_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("sih_pdhg_solve", "sih_pdhg_solve_ex", "sih_pdhg_is_cuda_available", "sih_pdhg_get_vram_info",
                 "sih_pdhg_launch_csr_spmv", "sih_pdhg_launch_csc_spmv", "sih_pdhg_launch_primal_update",
                 "sih_pdhg_launch_dual_update", "sih_pdhg_launch_restart", "sih_pdhg_launch_residuals"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from sih_pdhg import _lib

    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    """sizeof/offsetof from a C compile of the header equal the ctypes layouts."""
    from sih_pdhg import _lib
    from sih_pdhg.config import GpuPdhgConfig

    src = tmp_path / "sizes.c"
    fields = {"sih_pdhg_config": GpuPdhgConfig, "sih_pdhg_options": _lib.COptions,
              "sih_pdhg_result": _lib.CResult, "sih_pdhg_problem": _lib.CProblem,
              "sih_pdhg_launch_shape": _lib.CLaunchShape}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sih_pdhg.h"', "int main(void){"]
    for sname, cls in fields.items():
        lines.append(f'printf("{sname} %zu\\n", sizeof({sname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{sname}.{f} %zu\\n", offsetof({sname}, {f}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I", HEADER_DIR, str(src), "-o", str(exe)])
    out = dict(l.rsplit(" ", 1) for l in subprocess.check_output([str(exe)]).decode().split("\n") if l)
    for sname, cls in fields.items():
        assert int(out[sname]) == C.sizeof(cls), sname
        for f, _ in cls._fields_:
            assert int(out[f"{sname}.{f}"]) == getattr(cls, f).offset, f"{sname}.{f}"


def test_config_defaults_match_reference():
    """GpuPdhgConfig defaults of core/include/sih/gpu/gpu_solver.hpp:12-22."""
    from sih_pdhg import _lib
    from sih_pdhg.config import GpuPdhgConfig

    c = GpuPdhgConfig()
    _lib.load().sih_pdhg_config_default(C.byref(c))
    assert (c.max_iterations, c.check_frequency, c.enable_restart, c.enable_hybrid_polish) == (4000, 25, True, True)
    assert c.tol_primal == pytest.approx(1e-4) and c.tol_dual == pytest.approx(1e-4) and c.tol_gap == pytest.approx(1e-4)
    assert c.step_tau == 0.0 and c.step_sigma == 0.0
    py = GpuPdhgConfig()
    assert bytes(py) == bytes(c)


def test_invalid_arguments_rejected_before_device_work():
    """Malformed input returns SIH_PDHG_ERR_INVALID_ARGUMENT with a message, GPU or not."""
    import sih_pdhg
    from sih_pdhg import _lib
    from sih_pdhg.generators import small_random_lp

    p = small_random_lp(20, 40, 3, 0)
    bad = small_random_lp(20, 40, 3, 0)
    bad.A._ri = bad.A._ri.copy()
    bad.A._ri[5] = 10_000
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.solve_gpu_pdhg(bad)
    assert e.value.code == 1 and "csc_row_ind" in str(e.value)
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.solve_gpu_pdhg(p, sih_pdhg.GpuPdhgConfig(check_frequency=0))
    assert e.value.code == 1
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.GpuSolver.solve_ex(p, None, algorithm=7)
    assert e.value.code == 1


def test_no_device_is_an_error_not_a_fallback():
    import sih_pdhg
    from sih_pdhg.generators import small_random_lp

    if sih_pdhg.GpuSolver.is_cuda_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.solve_gpu_pdhg(small_random_lp(20, 40, 3, 0))
    assert e.value.code == 2


def test_generators_are_deterministic():
    from sih_pdhg.generators import small_random_lp, zipf_lp

    a, b = small_random_lp(300, 700, 5, 3), small_random_lp(300, 700, 5, 3)
    np.testing.assert_array_equal(a.A.csc_row_ind(), b.A.csc_row_ind())
    np.testing.assert_array_equal(a.c, b.c)
    z = zipf_lp(5000, 10000, 120000, seed=1)
    cnt = np.diff(z.A.csc_col_ptr())
    assert z.num_nonzeros() == 120000 and cnt.min() >= 2 and cnt.max() <= 2000
    # rows distinct within a column and sorted
    for j in range(0, 10000, 997):
        r = z.A.csc_row_ind()[z.A.csc_col_ptr()[j]:z.A.csc_col_ptr()[j + 1]]
        assert np.all(np.diff(r) > 0)
    # CSR holds the same entries
    x = np.random.default_rng(0).standard_normal(10000)
    dense_ax = z.A.mat_vec(x)
    cols = np.repeat(np.arange(10000), cnt)
    ref = np.bincount(z.A.csc_row_ind(), weights=z.A.csc_values() * x[cols], minlength=5000)
    np.testing.assert_allclose(dense_ax, ref, rtol=1e-12, atol=1e-12)


def test_adjoint_host_path_runs_without_a_device():
    """The adjoint's host part (validation, basis, layout) runs before the
    device check; without a GPU the call ends with the no-device status."""
    import sih_pdhg
    from sih_pdhg.generators import small_random_lp

    p = small_random_lp(60, 150, 4, 2)
    rng = np.random.default_rng(0)
    x = np.clip(rng.uniform(0, 5, 150), p.col_lower, p.col_upper)
    y = rng.standard_normal(60)
    if sih_pdhg.GpuSolver.is_cuda_available():
        pytest.skip("a device is present")
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.adjoint_batch([p], [x], [y], [np.ones(150)])
    assert e.value.code == 2
    with pytest.raises(sih_pdhg.SihPdhgError):
        sih_pdhg.adjoint_batch([p], [x[:10]], [y], [np.ones(150)])


def test_polish_host_path_runs_without_a_device():
    import sih_pdhg
    from sih_pdhg.generators import small_random_lp

    p = small_random_lp(60, 150, 4, 2)
    rng = np.random.default_rng(0)
    x = np.clip(rng.uniform(0, 5, 150), p.col_lower, p.col_upper)
    y = rng.standard_normal(60)
    if sih_pdhg.GpuSolver.is_cuda_available():
        pytest.skip("a device is present")
    with pytest.raises(sih_pdhg.SihPdhgError) as e:
        sih_pdhg.polish_batch([p], [x], [y])
    assert e.value.code == 2


C_CLIENT = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "sih_pdhg.h"

int main(int argc, char** argv) {
    sih_pdhg_mps* mps = NULL;
    if (sih_pdhg_read_mps(argv[1], &mps) != SIH_PDHG_OK) { printf("read %s\n", sih_pdhg_last_error()); return 1; }
    sih_pdhg_problem p;
    const char* name = NULL;
    int64_t ints = -1;
    if (sih_pdhg_mps_view(mps, &p, &name, &ints) != SIH_PDHG_OK) return 2;
    printf("problem %s %lld %lld %lld %lld %d %g\n", name, (long long)p.num_rows, (long long)p.num_cols,
           (long long)p.num_nonzeros, (long long)ints, p.sense, p.obj_offset);
    sih_pdhg_config cfg;
    sih_pdhg_config_default(&cfg);
    sih_pdhg_options opt;
    sih_pdhg_options_default(&opt);
    opt.algorithm = SIH_PDHG_ALGO_MIXED;
    double* x = calloc((size_t)p.num_cols, sizeof(double));
    double* y = calloc((size_t)p.num_rows, sizeof(double));
    sih_pdhg_result r = {0};
    r.x = x;
    r.row_duals = y;
    int rc = sih_pdhg_solve_ex(&p, &cfg, &opt, &r);
    printf("solve %d %d %.9g\n", rc, r.status, r.primal_objective);
    sih_pdhg_result rp = {0};
    rp.x = x;
    rp.row_duals = y;
    rc = sih_pdhg_solve(&p, &cfg, &rp); /* the GpuSolver::solve_pdhg drop-in (reference algorithm) */
    printf("plain %d %d %.9g %lld %.9g %.9g\n", rc, rp.status, rp.primal_objective, (long long)rp.iterations,
           x[0], x[1]);
    free(x);
    free(y);
    sih_pdhg_mps_free(mps);
    return 0;
}
"""


def _run_c_client(tmp_path):
    """Compiles the C client against the library and runs it on a toy MPS file:
    min -x1 - 2 x2, x1 + x2 <= 4, x1 - x2 <= -1, x >= 0 (optimum -8 at (0, 4))."""
    from sih_pdhg import _lib

    lib_path = _lib.LIB_PATH
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", HEADER_DIR, str(src), "-o", str(exe),
                           lib_path, f"-Wl,-rpath,{os.path.dirname(lib_path)}", "-lm"])
    mps = tmp_path / "toy.mps"
    mps.write_text("NAME toy\nROWS\n N  OBJ\n L  R1\n L  R2\nCOLUMNS\n    X1  OBJ  -1.0  R1  1.0\n"
                   "    X1  R2  1.0\n    X2  OBJ  -2.0  R1  1.0\n    X2  R2  -1.0\nRHS\n    RHS  R1  4.0  R2  -1.0\n"
                   "ENDATA\n")
    out = subprocess.run([str(exe), str(mps)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = dict(l.split(" ", 1) for l in out.stdout.splitlines())
    assert lines["problem"] == "toy 2 2 4 0 1 0"
    return lines


def test_plain_c_client_reads_mps_and_calls_the_solver(tmp_path):
    """The ABI from C (no C++ or Python in between): read an MPS file into a
    sih_pdhg_problem view and hand it to sih_pdhg_solve_ex and sih_pdhg_solve.
    Without a device both return SIH_PDHG_ERR_NO_DEVICE after the problem was
    accepted (no CPU fallback)."""
    from sih_pdhg import _lib

    lib = _lib.load()
    if lib.sih_pdhg_is_cuda_available():
        pytest.skip("device present: the GPU-marked test below runs the solves")
    lines = _run_c_client(tmp_path)
    assert lines["solve"].split()[0] == "2"
    assert lines["plain"].split()[0] == "2"


@pytest.mark.gpu
def test_plain_c_client_solves_on_the_gpu(tmp_path):
    """Same C client on a GPU: the mixed solve and the drop-in for
    GpuSolver::solve_pdhg (reference algorithm and config defaults) both reach
    the optimum -8 at (0, 4)."""
    lines = _run_c_client(tmp_path)
    rc, status, obj = lines["solve"].split()
    assert int(rc) == 0 and int(status) == 0, lines["solve"]
    assert abs(float(obj) - (-8.0)) <= 1e-3
    rc, status, obj, iters, x0, x1 = lines["plain"].split()
    assert int(rc) == 0 and int(status) == 0, lines["plain"]
    assert abs(float(obj) - (-8.0)) <= 1e-3 and abs(float(x0)) <= 1e-3 and abs(float(x1) - 4.0) <= 1e-3

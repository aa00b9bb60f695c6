"""ctypes loader for the C oracle (oracle/pdhg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py, never by the shipped package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-ffp-contract=off keeps float ops unfused)."""
    srcs = [os.path.join(HERE, "pdhg_oracle.c"), os.path.join(HERE, "pdlp_oracle.c")]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.abspath(__file__)])
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               *srcs, "-o", LIB_PATH, "-lm"])
    return LIB_PATH


def reference_dir():
    """Directory of the reference sources as the build recipe oracle/ref_build.sh
    resolves it (SIH_REFERENCE_DIR or the recipe's default), or None where the
    sources are absent (the GPU machine)."""
    out = subprocess.run(["bash", os.path.join(HERE, "ref_build.sh"), "--print-dir"], capture_output=True, text=True)
    d = out.stdout.strip()
    return d if out.returncode == 0 and d else None


class OracleConfig(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("tol_primal", C.c_float), ("tol_dual", C.c_float),
                ("tol_gap", C.c_float), ("check_frequency", C.c_int32), ("step_tau", C.c_float),
                ("step_sigma", C.c_float), ("enable_restart", C.c_uint8), ("enable_hybrid_polish", C.c_uint8)]


class OraclePlainInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int64), ("primal_objective", C.c_double),
                ("last_norm_p", C.c_float), ("last_norm_d", C.c_float), ("best_combined", C.c_float),
                ("checks", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def config_from(cfg) -> OracleConfig:
    """Copy the fields of any GpuPdhgConfig-like object."""
    o = OracleConfig()
    for name, _ in OracleConfig._fields_:
        v = getattr(cfg, name)
        setattr(o, name, int(v) if name in ("max_iterations", "check_frequency", "enable_restart",
                                            "enable_hybrid_polish") else float(v))
    return o


def plain_pdhg(problem, cfg, threads: int = 0):
    """Reference-semantics plain FP32 PDHG on the CPU.  Returns (x, y, info dict)."""
    A = problem.A
    m, n = problem.num_rows(), problem.num_cols()
    x = np.zeros(n)
    y = np.zeros(m)
    info = OraclePlainInfo()
    oc = config_from(cfg)
    arrs = [np.ascontiguousarray(a) for a in (A.csc_col_ptr(), A.csc_row_ind(), A.csc_values(), problem.c,
                                              problem.col_lower, problem.col_upper, problem.row_lower,
                                              problem.row_upper)]
    rc = lib().oracle_plain_pdhg(C.c_int64(m), C.c_int64(n), _p(arrs[0], C.c_int64), _p(arrs[1], C.c_int64),
                                 _p(arrs[2], C.c_double), _p(arrs[3], C.c_double), _p(arrs[4], C.c_double),
                                 _p(arrs[5], C.c_double), _p(arrs[6], C.c_double), _p(arrs[7], C.c_double),
                                 C.byref(oc), _p(x, C.c_double), _p(y, C.c_double), C.byref(info), C.c_int(threads))
    if rc != 0:
        raise ValueError("oracle_plain_pdhg rejected its arguments")
    return x, y, {k: getattr(info, k) for k, _ in OraclePlainInfo._fields_}


def kkt(problem, x, y):
    """FP64 relative KKT of (x, y) with y in the PDHG sign.  Returns dict."""
    A = problem.A
    out = np.zeros(6)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    lib().oracle_kkt(C.c_int64(problem.num_rows()), C.c_int64(problem.num_cols()), _p(A.csc_col_ptr(), C.c_int64),
                     _p(A.csc_row_ind(), C.c_int64), _p(A.csc_values(), C.c_double), _p(problem.c, C.c_double),
                     _p(problem.col_lower, C.c_double), _p(problem.col_upper, C.c_double),
                     _p(problem.row_lower, C.c_double), _p(problem.row_upper, C.c_double), _p(x, C.c_double),
                     _p(y, C.c_double), _p(out, C.c_double))
    return dict(rel_primal=out[0], rel_dual=out[1], rel_gap=out[2], primal_obj=out[3], dual_obj=out[4],
                abs_primal=out[5])


def csr_spmv_f32(rp, ci, v, x):
    rp, ci = np.ascontiguousarray(rp, np.int32), np.ascontiguousarray(ci, np.int32)
    v, x = np.ascontiguousarray(v, np.float32), np.ascontiguousarray(x, np.float32)
    y = np.zeros(rp.shape[0] - 1, np.float32)
    lib().oracle_csr_spmv_f32(C.c_int(y.shape[0]), _p(rp, C.c_int), _p(ci, C.c_int), _p(v, C.c_float),
                              _p(x, C.c_float), _p(y, C.c_float))
    return y


def csc_spmv_f32(cp, ri, v, y):
    cp, ri = np.ascontiguousarray(cp, np.int32), np.ascontiguousarray(ri, np.int32)
    v, y = np.ascontiguousarray(v, np.float32), np.ascontiguousarray(y, np.float32)
    z = np.zeros(cp.shape[0] - 1, np.float32)
    lib().oracle_csc_spmv_f32(C.c_int(z.shape[0]), _p(cp, C.c_int), _p(ri, C.c_int), _p(v, C.c_float),
                              _p(y, C.c_float), _p(z, C.c_float))
    return z


def primal_update_f32(tau, c, aty, l, u, x):
    f = lambda a: np.ascontiguousarray(a, np.float32)
    tau, c, aty, l, u = map(f, (tau, c, aty, l, u))
    x = f(x).copy()
    xbar = np.zeros_like(x)
    lib().oracle_primal_update_f32(C.c_int(x.shape[0]), _p(tau, C.c_float), _p(c, C.c_float), _p(aty, C.c_float),
                                   _p(l, C.c_float), _p(u, C.c_float), _p(x, C.c_float), _p(xbar, C.c_float))
    return x, xbar


def dual_update_f32(sigma, axbar, rl, ru, y):
    f = lambda a: np.ascontiguousarray(a, np.float32)
    sigma, axbar, rl, ru = map(f, (sigma, axbar, rl, ru))
    y = f(y).copy()
    lib().oracle_dual_update_f32(C.c_int(y.shape[0]), _p(sigma, C.c_float), _p(axbar, C.c_float),
                                 _p(rl, C.c_float), _p(ru, C.c_float), _p(y, C.c_float))
    return y


class PdlpOpts(C.Structure):
    _fields_ = [("ruiz_iterations", C.c_int32), ("pock_chambolle", C.c_int32), ("eval_frequency", C.c_int32),
                ("enable_restart", C.c_int32), ("max_attempts", C.c_int64), ("tol_p", C.c_double),
                ("tol_d", C.c_double), ("tol_g", C.c_double), ("beta_suff", C.c_double), ("beta_nec", C.c_double),
                ("beta_art", C.c_double), ("weight_smoothing", C.c_double), ("fp32_bits", C.c_int32)]


class PdlpInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("out_sel", C.c_int32), ("attempts", C.c_int64), ("steps", C.c_int64),
                ("rejections", C.c_int64), ("restarts", C.c_int64), ("evals", C.c_int64), ("eta", C.c_double),
                ("omega", C.c_double), ("rel_p", C.c_double), ("rel_d", C.c_double), ("rel_g", C.c_double),
                ("pobj", C.c_double), ("dobj", C.c_double)]


def pdlp_solve(problem, max_attempts=100000, tol=1e-4, tol_p=None, tol_d=None, tol_g=None, eval_frequency=64,
               ruiz_iterations=10, pock_chambolle=1, enable_restart=1, fp32_bits=0, weight_smoothing=0.5,
               restart_sufficient=0.2, restart_necessary=0.8, restart_artificial=0.36):
    """FP64 restarted adaptive PDHG (the algorithm of the mixed CUDA path, with its
    default options: primal weight smoothing 0.5, restart thresholds 0.2 / 0.8 / 0.36).
    Returns (x, y_pdhg, info dict); a maximization problem is solved as min -c."""
    A = problem.A
    m, n = problem.num_rows(), problem.num_cols()
    o = PdlpOpts(ruiz_iterations, pock_chambolle, eval_frequency, enable_restart, max_attempts,
                 tol if tol_p is None else tol_p, tol if tol_d is None else tol_d, tol if tol_g is None else tol_g,
                 restart_sufficient, restart_necessary, restart_artificial, weight_smoothing, fp32_bits)
    c = np.ascontiguousarray(problem.c * (1 if int(problem.sense) == 1 else -1), dtype=np.float64)
    x = np.zeros(n)
    y = np.zeros(m)
    info = PdlpInfo()
    lib().pdlp_oracle_solve(C.c_int64(m), C.c_int64(n), _p(A.csc_col_ptr(), C.c_int64), _p(A.csc_row_ind(), C.c_int64),
                            _p(A.csc_values(), C.c_double), _p(c, C.c_double), _p(problem.col_lower, C.c_double),
                            _p(problem.col_upper, C.c_double), _p(problem.row_lower, C.c_double),
                            _p(problem.row_upper, C.c_double), C.byref(o), _p(x, C.c_double), _p(y, C.c_double),
                            C.byref(info))
    return x, y, {k: getattr(info, k) for k, _ in PdlpInfo._fields_}


def plain_prepare(problem):
    """FP32/int32 arrays of the reference algorithm for oracle_plain_iterations
    (the CPU baseline's timing loop).  Step sizes 0.95 / max(1, sum |a|) as in
    gpu_solver.cpp:128-151 (summed by numpy here: the sample is a timing sample)."""
    A = problem.A
    m, n = problem.num_rows(), problem.num_cols()
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    cp, ri, cv = i32(A.csc_col_ptr()), i32(A.csc_row_ind()), f32(A.csc_values())
    rp, ci, rv = i32(A.csr_row_ptr()), i32(A.csr_col_ind()), f32(A.csr_values())
    cols = np.repeat(np.arange(n), np.diff(cp))
    rows = np.repeat(np.arange(m), np.diff(rp))
    colsum = np.bincount(cols, weights=np.abs(cv), minlength=n).astype(np.float32)
    rowsum = np.bincount(rows, weights=np.abs(rv), minlength=m).astype(np.float32)
    l, u = f32(problem.col_lower), f32(problem.col_upper)
    x = np.maximum(l, np.minimum(u, np.float32(0)))
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    return dict(m=m, n=n, cp=cp, ri=ri, cv=cv, rp=rp, ci=ci, rv=rv, c=f32(problem.c), l=l, u=u,
                cv64=f64(A.csc_values()), rv64=f64(A.csr_values()), c64=f64(problem.c), l64=f64(problem.col_lower),
                u64=f64(problem.col_upper), rl64=f64(problem.row_lower), ru64=f64(problem.row_upper),
                rl=f32(problem.row_lower), ru=f32(problem.row_upper),
                tau=(np.float32(0.95) / np.maximum(np.float32(1), colsum)).astype(np.float32),
                sigma=(np.float32(0.95) / np.maximum(np.float32(1), rowsum)).astype(np.float32),
                x=x.copy(), xbar=x.copy(), y=np.zeros(m, np.float32), aty=np.zeros(n, np.float32),
                axbar=np.zeros(m, np.float32))


def plain_iterations(d, iters: int, threads: int = 0) -> None:
    """Runs `iters` reference PDHG iterations (the four kernels of
    core/src/gpu/cuda_pdhg.cu:14-103, OpenMP) on prepared arrays, in place."""
    F, I = C.c_float, C.c_int
    lib().oracle_plain_iterations(
        C.c_int(d["m"]), C.c_int(d["n"]), _p(d["cp"], I), _p(d["ri"], I), _p(d["cv"], F), _p(d["rp"], I),
        _p(d["ci"], I), _p(d["rv"], F), _p(d["c"], F), _p(d["l"], F), _p(d["u"], F), _p(d["rl"], F),
        _p(d["ru"], F), _p(d["tau"], F), _p(d["sigma"], F), _p(d["x"], F), _p(d["xbar"], F), _p(d["y"], F),
        _p(d["aty"], F), _p(d["axbar"], F), C.c_int(iters), C.c_int(threads))


def plain_solve_kkt(d, tol: float, eval_every: int = 100, max_iters: int = 1_000_000, threads: int = 0) -> dict:
    """The reference algorithm (plain FP32 PDHG, core/src/gpu/cuda_pdhg.cu:14-103
    with the steps of gpu_solver.cpp:128-151) from its initial point until the
    FP64 relative KKT of the current (x, y) is <= tol (checked every
    `eval_every` iterations; the reference's own stopping test off), OpenMP.
    `d` comes from plain_prepare.  Returns iterations and the KKT triple."""
    F, I, D = C.c_float, C.c_int, C.c_double
    out = np.zeros(4)
    rc = lib().oracle_plain_solve_kkt(
        C.c_int(d["m"]), C.c_int(d["n"]), _p(d["cp"], I), _p(d["ri"], I), _p(d["cv"], F), _p(d["cv64"], D),
        _p(d["rp"], I), _p(d["ci"], I), _p(d["rv"], F), _p(d["rv64"], D), _p(d["c64"], D), _p(d["l64"], D),
        _p(d["u64"], D), _p(d["rl64"], D), _p(d["ru64"], D), C.c_double(tol), C.c_int(eval_every),
        C.c_int(max_iters), C.c_int(threads), _p(out, D))
    if rc != 0:
        raise ValueError("oracle_plain_solve_kkt rejected its arguments")
    return dict(iterations=int(out[0]), rel_primal=float(out[1]), rel_dual=float(out[2]), rel_gap=float(out[3]))


def basis_guess(problem, x, row_activity):
    """Basis guess of the reference's hybrid polish (core/src/gpu/gpu_solver.cpp:332-395):
    distance of every column value / row activity to its nearer finite bound
    (bounds beyond +-1e15 absent: distance 1e30), the m largest Basic (0), the
    rest AtLower (1) / AtUpper (2) by the nearer bound (AtLower on a tie); equal
    distances in candidate order (columns, then rows), i.e. a stable descending
    sort.  Returns (col_status, row_status) int8 arrays."""
    n, m = problem.num_cols(), problem.num_rows()
    v = np.concatenate([np.asarray(x, dtype=np.float64), np.asarray(row_activity, dtype=np.float64)])
    lo = np.concatenate([problem.col_lower, problem.row_lower]).astype(np.float64)
    hi = np.concatenate([problem.col_upper, problem.row_upper]).astype(np.float64)
    dl = np.where(lo > -1e15, np.maximum(0.0, v - lo), 1e30)
    du = np.where(hi < 1e15, np.maximum(0.0, hi - v), 1e30)
    d = np.minimum(dl, du)
    status = np.where(dl <= du, 1, 2).astype(np.int8)
    status[np.argsort(-d, kind="stable")[:m]] = 0
    return status[:n], status[n:]

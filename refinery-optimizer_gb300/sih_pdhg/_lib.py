"""ctypes binding of the engine's C ABI (include/sih_pdhg.h).

The library is ``refinery-optimizer_gb300/_build/libsih_pdhg.so`` built by
``refinery-optimizer_gb300/build.py``.  There is no fallback: if the library is
missing, loading raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .config import GpuPdhgConfig

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("SIH_PDHG_LIB") or os.path.join(PKG_DIR, "_build", "libsih_pdhg.so")

OK = 0
ABI_VERSION = 2  # SIH_PDHG_ABI_VERSION of include/sih_pdhg.h that these ctypes layouts mirror
ERR_NAMES = {1: "invalid argument", 2: "no CUDA device", 3: "CUDA error", 4: "out of memory", 5: "unsupported"}

ALGO_PLAIN = 0
ALGO_MIXED = 1


class SihPdhgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sih_pdhg error {code} ({ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


class CProblem(C.Structure):
    _fields_ = [("num_rows", C.c_int64), ("num_cols", C.c_int64), ("num_nonzeros", C.c_int64),
                ("csc_col_ptr", C.c_void_p), ("csc_row_ind", C.c_void_p), ("csc_values", C.c_void_p),
                ("csr_row_ptr", C.c_void_p), ("csr_col_ind", C.c_void_p), ("csr_values", C.c_void_p),
                ("c", C.c_void_p), ("col_lower", C.c_void_p), ("col_upper", C.c_void_p),
                ("row_lower", C.c_void_p), ("row_upper", C.c_void_p), ("sense", C.c_int32),
                ("obj_offset", C.c_double)]


class COptions(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("algorithm", C.c_int32), ("ruiz_iterations", C.c_int32),
                ("pock_chambolle", C.c_int32), ("eval_frequency", C.c_int32), ("compensated", C.c_int32),
                ("dual_sign", C.c_int32), ("use_graph", C.c_int32), ("autotune", C.c_int32),
                ("verbose", C.c_int32), ("time_limit_sec", C.c_double), ("restart_sufficient", C.c_double),
                ("restart_necessary", C.c_double), ("restart_artificial", C.c_double),
                ("primal_weight_smoothing", C.c_double), ("exact_arithmetic", C.c_int32),
                ("lanes_csr", C.c_int32), ("lanes_csc", C.c_int32), ("heavy_factor", C.c_int32),
                ("tile_nnz", C.c_int32), ("reorder", C.c_int32), ("staged_kib", C.c_int32),
                ("persistent", C.c_int32), ("packed", C.c_int32), ("reserved2", C.c_int32)]


class CLaunchShape(C.Structure):
    _fields_ = [("task_nnz", C.c_int32), ("row_lanes", C.c_int32), ("col_lanes", C.c_int32),
                ("staged_x", C.c_int32), ("staged_y", C.c_int32), ("persistent", C.c_int32), ("grid", C.c_int32),
                ("tuned", C.c_int32), ("packed", C.c_int32), ("reserved", C.c_int32)]


class CAdjointOptions(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("reserved", C.c_int32), ("tolerance", C.c_double),
                ("max_iterations", C.c_int64)]


class CAdjointInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved", C.c_int32), ("iterations", C.c_int64), ("residual", C.c_double),
                ("free_columns", C.c_int64), ("active_rows", C.c_int64)]


class CPolishInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved", C.c_int32), ("iterations", C.c_int64),
                ("primal_residual", C.c_double), ("dual_residual", C.c_double), ("primal_violation", C.c_double),
                ("dual_violation", C.c_double), ("free_columns", C.c_int64), ("active_rows", C.c_int64)]


class CResult(C.Structure):
    _fields_ = [("x", C.c_void_p), ("row_duals", C.c_void_p), ("slack", C.c_void_p),
                ("reduced_costs", C.c_void_p), ("status", C.c_int32), ("reserved0", C.c_int32),
                ("iterations", C.c_int64), ("primal_objective", C.c_double), ("dual_bound", C.c_double),
                ("rel_primal", C.c_double), ("rel_dual", C.c_double), ("rel_gap", C.c_double),
                ("ref_primal", C.c_double), ("ref_dual", C.c_double), ("time_wall_sec", C.c_double),
                ("time_solver_sec", C.c_double), ("restarts", C.c_int64), ("step_rejections", C.c_int64),
                ("final_step", C.c_double), ("final_primal_weight", C.c_double), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("kernel_launches", C.c_uint64)]


_lib = None


def load() -> C.CDLL:
    """Load the engine library (raises RuntimeError if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python refinery-optimizer_gb300/build.py` "
                           "(the engine has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
    lib.sih_pdhg_abi_version.restype = i32
    if lib.sih_pdhg_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{LIB_PATH} has ABI version {lib.sih_pdhg_abi_version()}, this binding expects "
                           f"{ABI_VERSION}: rebuild the library")
    lib.sih_pdhg_last_error.restype = C.c_char_p
    lib.sih_pdhg_is_cuda_available.restype = i32
    lib.sih_pdhg_get_vram_info.argtypes = [C.POINTER(C.c_uint64)] * 3
    lib.sih_pdhg_solve.argtypes = [C.POINTER(CProblem), C.POINTER(GpuPdhgConfig), C.POINTER(CResult)]
    lib.sih_pdhg_solve_ex.argtypes = [C.POINTER(CProblem), C.POINTER(GpuPdhgConfig), C.POINTER(COptions),
                                      C.POINTER(CResult)]
    lib.sih_pdhg_options_default.argtypes = [C.POINTER(COptions)]
    lib.sih_pdhg_config_default.argtypes = [C.POINTER(GpuPdhgConfig)]
    lib.sih_pdhg_launch_csr_spmv.argtypes = [i32, vp, vp, vp, vp, vp, vp]
    lib.sih_pdhg_launch_csc_spmv.argtypes = [i32, vp, vp, vp, vp, vp, vp]
    lib.sih_pdhg_launch_primal_update.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.sih_pdhg_launch_dual_update.argtypes = [i32, vp, vp, vp, vp, vp, vp]
    lib.sih_pdhg_launch_restart.argtypes = [i32, vp, vp, vp]
    lib.sih_pdhg_launch_residuals.argtypes = [i32, i32] + [vp] * 12
    lib.sih_pdhg_create.argtypes = [C.POINTER(CProblem), C.c_int32, C.POINTER(GpuPdhgConfig), C.POINTER(COptions),
                                    C.POINTER(C.c_void_p)]
    lib.sih_pdhg_run.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.sih_pdhg_get_result.argtypes = [C.c_void_p, C.c_int32, C.POINTER(CResult)]
    lib.sih_pdhg_time_kernels.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.sih_pdhg_set_start.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_double]
    lib.sih_pdhg_get_task_nnz.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    lib.sih_pdhg_basis_guess.argtypes = [C.POINTER(CProblem), vp, vp, vp, vp]
    lib.sih_pdhg_get_launch_shape.argtypes = [C.c_void_p, C.POINTER(CLaunchShape)]
    lib.sih_pdhg_check_grid_barrier.argtypes = [i32, i32, i32, C.c_double, C.POINTER(C.c_int32),
                                                C.POINTER(C.c_int32)]
    lib.sih_pdhg_adjoint_options_default.argtypes = [C.c_void_p]
    lib.sih_pdhg_adjoint_options_default.restype = None
    pp = C.POINTER(C.c_void_p)
    lib.sih_pdhg_adjoint_batch.argtypes = [C.c_void_p, C.c_int32, pp, pp, pp, pp, pp, pp, pp, pp, C.c_void_p,
                                           C.c_void_p]
    lib.sih_pdhg_polish_batch.argtypes = [C.c_void_p, C.c_int32, pp, pp, pp, pp, C.c_void_p, C.c_void_p]
    lib.sih_pdhg_destroy.argtypes = [C.c_void_p]
    lib.sih_pdhg_destroy.restype = None
    lib.sih_pdhg_check_norms_noalloc.argtypes = [i32, i32, i32] + [vp] * 14 + [C.c_float, C.c_float, vp, vp]
    lib.sih_pdhg_solve_batch.argtypes = [C.POINTER(CProblem), C.c_int32, C.POINTER(GpuPdhgConfig),
                                         C.POINTER(COptions), C.POINTER(CResult)]
    lib.sih_pdhg_read_mps.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    lib.sih_pdhg_read_mps_text.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_void_p)]
    lib.sih_pdhg_mps_view.argtypes = [C.c_void_p, C.POINTER(CProblem), C.POINTER(C.c_char_p),
                                      C.POINTER(C.c_int64)]
    lib.sih_pdhg_mps_free.argtypes = [C.c_void_p]
    lib.sih_pdhg_mps_free.restype = None
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != OK:
        raise SihPdhgError(rc, load().sih_pdhg_last_error().decode(errors="replace"))


def default_options(**kw) -> COptions:
    o = COptions()
    load().sih_pdhg_options_default(C.byref(o))
    for k, v in kw.items():
        if not any(k == f[0] for f in COptions._fields_):
            raise AttributeError(f"unknown option {k!r}")
        setattr(o, k, v)
    return o


def _ptr(a):
    return None if a is None else a.ctypes.data


def c_problem(problem):
    """CProblem view of a sih_pdhg.Problem (keeps the arrays alive in `keep`)."""
    A = problem.A
    csr = (A.csr_row_ptr(), A.csr_col_ind(), A.csr_values()) if A.has_csr() else (None, None, None)
    keep = [None if a is None else np.ascontiguousarray(a)
            for a in (A.csc_col_ptr(), A.csc_row_ind(), A.csc_values(), *csr, problem.c, problem.col_lower,
                      problem.col_upper, problem.row_lower, problem.row_upper)]
    cp = CProblem(problem.num_rows(), problem.num_cols(), problem.num_nonzeros(), *[_ptr(a) for a in keep],
                  int(problem.sense), float(problem.obj_offset))
    return cp, keep

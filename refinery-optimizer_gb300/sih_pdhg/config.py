"""Solver configuration structs.

``GpuPdhgConfig`` has the fields, defaults and meaning of the reference's
``sih::gpu::GpuPdhgConfig`` (core/include/sih/gpu/gpu_solver.hpp:12-22) and the
same C layout (see include/sih_pdhg.h).  ``PdhgOptions`` holds the settings of
the added entry points (precision/algorithm, scaling, restarts, batching).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass


class GpuPdhgConfig(C.Structure):
    """Layout-identical to ``sih::gpu::GpuPdhgConfig`` (int, 3 float, int, 2 float, 2 bool)."""
    _fields_ = [("max_iterations", C.c_int32), ("tol_primal", C.c_float), ("tol_dual", C.c_float),
                ("tol_gap", C.c_float), ("check_frequency", C.c_int32), ("step_tau", C.c_float),
                ("step_sigma", C.c_float), ("enable_restart", C.c_bool), ("enable_hybrid_polish", C.c_bool)]

    def __init__(self, **kw):
        super().__init__()
        self.max_iterations = 4000
        self.tol_primal = 1e-4
        self.tol_dual = 1e-4
        self.tol_gap = 1e-4
        self.check_frequency = 25
        self.step_tau = 0.0  # 0 = automatic
        self.step_sigma = 0.0
        self.enable_restart = True
        self.enable_hybrid_polish = True
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"GpuPdhgConfig has no field {k!r}")
            setattr(self, k, v)

    def __repr__(self) -> str:
        return "GpuPdhgConfig(" + ", ".join(f"{k}={getattr(self, k)!r}" for k, _ in self._fields_) + ")"

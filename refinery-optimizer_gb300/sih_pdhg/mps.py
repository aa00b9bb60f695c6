"""MPS text of a Problem (free format), the counterpart of ``read_mps``.

Rows: equality ``E``, one-sided ``L`` / ``G``, two-sided ``G`` with a range
(``[rhs, rhs + R]``), free rows ``L`` with an infinite right-hand side.  The
objective offset is written as the objective row's RHS (``-offset``, the
sign the reference's reader applies, core/src/io/mps_io.cpp:224-226).  Bounds
use FX, FR, MI + UP, LO and UP.  Numbers are written with ``repr`` so that
``strtod`` reads back the same doubles; ranged rows come back as
``rhs + (upper - lower)``, which may differ from ``upper`` in the last bit.
"""
from __future__ import annotations

import math

import numpy as np

from .problem import ObjectiveSense, Problem


def _num(v: float) -> str:
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return repr(float(v))


def mps_text(problem: Problem) -> str:
    p = problem
    m, n = p.num_rows(), p.num_cols()
    rl, ru, lo, up = p.row_lower, p.row_upper, p.col_lower, p.col_upper
    out = [f"NAME {p.name or 'problem'}"]
    if int(p.sense) == int(ObjectiveSense.Maximize):
        out += ["OBJSENSE", "    MAX"]
    out.append("ROWS")
    out.append(" N  OBJ")
    rhs, rng = [], []
    for i in range(m):
        fl, fu = math.isfinite(rl[i]), math.isfinite(ru[i])
        if fl and fu and rl[i] == ru[i]:
            out.append(f" E  R{i}")
            rhs.append((i, rl[i]))
        elif fl and fu:
            out.append(f" G  R{i}")
            rhs.append((i, rl[i]))
            rng.append((i, ru[i] - rl[i]))
        elif fl:
            out.append(f" G  R{i}")
            rhs.append((i, rl[i]))
        elif fu:
            out.append(f" L  R{i}")
            rhs.append((i, ru[i]))
        else:
            out.append(f" L  R{i}")
            rhs.append((i, math.inf))
    out.append("COLUMNS")
    cp, ri, cv = p.A.csc_col_ptr(), p.A.csc_row_ind(), p.A.csc_values()
    for j in range(n):
        out.append(f"    C{j}  OBJ  {_num(p.c[j])}")
        for k in range(int(cp[j]), int(cp[j + 1])):
            out.append(f"    C{j}  R{int(ri[k])}  {_num(cv[k])}")
    out.append("RHS")
    if p.obj_offset != 0.0:
        out.append(f"    RHS  OBJ  {_num(-p.obj_offset)}")
    out += [f"    RHS  R{i}  {_num(v)}" for i, v in rhs if v != 0.0]
    if rng:
        out.append("RANGES")
        out += [f"    RNG  R{i}  {_num(v)}" for i, v in rng]
    out.append("BOUNDS")
    for j in range(n):
        l, u = float(lo[j]), float(up[j])
        if l == u:
            out.append(f" FX BND  C{j}  {_num(l)}")
        elif math.isinf(l) and math.isinf(u):
            out.append(f" FR BND  C{j}")
        elif math.isinf(l):
            out.append(f" MI BND  C{j}")
            out.append(f" UP BND  C{j}  {_num(u)}")
        else:
            if l != 0.0:
                out.append(f" LO BND  C{j}  {_num(l)}")
            if not math.isinf(u):
                out.append(f" UP BND  C{j}  {_num(u)}")
    out.append("ENDATA")
    return "\n".join(out) + "\n"


def write_mps(problem: Problem, path) -> None:
    """Write ``problem`` as a free-format MPS file."""
    with open(path, "w") as f:
        f.write(mps_text(problem))


def same_problem(a: Problem, b: Problem, bound_rtol: float = 0.0) -> None:
    """Raise AssertionError unless a and b hold the same LP (matrix, objective,
    bounds, sense, offset); row bounds compared with ``bound_rtol``."""
    np.testing.assert_array_equal(a.A.csc_col_ptr(), b.A.csc_col_ptr())
    np.testing.assert_array_equal(a.A.csc_row_ind(), b.A.csc_row_ind())
    np.testing.assert_array_equal(a.A.csc_values(), b.A.csc_values())
    np.testing.assert_array_equal(a.c, b.c)
    np.testing.assert_array_equal(a.col_lower, b.col_lower)
    np.testing.assert_array_equal(a.col_upper, b.col_upper)
    np.testing.assert_allclose(a.row_lower, b.row_lower, rtol=bound_rtol, atol=0)
    np.testing.assert_allclose(a.row_upper, b.row_upper, rtol=bound_rtol, atol=0)
    assert int(a.sense) == int(b.sense) and float(a.obj_offset) == float(b.obj_offset)

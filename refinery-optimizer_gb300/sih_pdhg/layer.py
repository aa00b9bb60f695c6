"""Differentiable LP layer: torch.autograd.Function over the GB300 engine.

    x = lp_layer(matrices, c, row_lower, row_upper, col_lower, col_upper)

Forward: one batched solve of the LPs
    min c_i^T x  s.t.  row_lower_i <= A_i x <= row_upper_i,  col_lower_i <= x <= col_upper_i
with the mixed-precision restarted adaptive PDHG (sih_pdhg_solve_batch), then
the basis polish (sih_pdhg_polish_batch): the layer returns the vertex of the
basis read off the PDHG point, the point whose neighbourhood the backward
differentiates, when that vertex is certified optimal (its bound violations and
wrong-sign reduced costs are at most ``certify_tol``, relative).  Otherwise the
basis was misread (near-degenerate variables that the FP32 PDHG point at its
tolerance cannot separate; measured on 20,000 x 50,000 LPs of 10 nonzeros per
column, where no basis read off a 1e-6 point was optimal): the instance returns
its PDHG point instead, which satisfies the LP to the solve's tolerance, a
``LPLayerWarning`` names the instances, and their gradients are those of the
basis that was read, an approximation.
Optimal values (return_objective=True): v* = c^T x* with gradients from the
duals by the envelope theorem (objective_gradients), exact at the returned
point and independent of the basis.
Backward of x*: the adjoint kernel (sih_pdhg_adjoint_batch): the active pattern of
the PDHG fixed point read off (x*, y*) as a basis, and B^T lambda = dL/dx_F
solved on the GPU by CGLS with the engine's SpMVs.  Gradients flow to the row
bounds and column bounds; the objective's implicit gradient is zero (an LP
solution is locally constant in c), so dL/dc is what the loss itself puts on c
(for L = |x* - t|^2 + lam c^T x*, that is lam x*).

Tensors are float64, shaped (batch, n) for c / col bounds and (batch, m) for
row bounds, on any device (the solve copies them to the host); infinite bounds
are +-inf.  The matrices (one sih_pdhg SparseMatrix per instance, all of the
same shape) are constants of the layer.
"""
from __future__ import annotations

import warnings
from typing import List, Optional

import numpy as np

from . import adjoint_batch, polish_batch, solve_batch
from .config import GpuPdhgConfig
from .problem import ObjectiveSense, Problem, SparseMatrix

try:
    import torch
except ImportError:  # the layer needs torch; the rest of the package does not
    torch = None


class LPLayerWarning(UserWarning):
    """Some instances of a layer call returned their PDHG point, not a certified vertex."""


def choose_outputs(sols, xs, ys, infos, certify_tol: float):
    """Per instance, the polished vertex and its duals when the polish certified
    the basis optimal, else the PDHG point and duals.  Returns (x list, y list,
    indices of the uncertified instances)."""
    x_out, y_out, bad = [], [], []
    for i, (s, x, y, info) in enumerate(zip(sols, xs, ys, infos)):
        ok = (info["status"] == 0 and info["primal_violation"] <= certify_tol
              and info["dual_violation"] <= certify_tol)
        x_out.append(x if ok else s.x)
        y_out.append(y if ok else s.row_duals)
        if not ok:
            bad.append(i)
    return x_out, y_out, bad


def objective_gradients(problem: Problem, x, y_pdhg) -> dict:
    """Gradient of the optimal value v = c^T x* of a minimisation LP with respect
    to its data, from a primal-dual optimal pair (the envelope theorem, i.e. LP
    sensitivity analysis; no linear system): dv/dc = x*, dv/d row bound = the
    simplex dual y = -y_pdhg (to row_lower where y > 0 or the row is an
    equality, to row_upper where y < 0), dv/d column bound = the reduced cost
    lambda = c - A^T y (to col_lower where lambda > 0, to col_upper where
    lambda < 0, finite bounds only).  Needs no basis, so it is as accurate as
    the PDHG point itself on LPs whose basis the polish cannot identify."""
    A = problem.A
    m, n = problem.num_rows(), problem.num_cols()
    y = -np.asarray(y_pdhg, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    cp, ri, cv = A.csc_col_ptr(), A.csc_row_ind(), A.csc_values()
    aty = np.zeros(n)
    cols = np.repeat(np.arange(n), np.diff(cp))
    np.add.at(aty, cols, cv * y[ri])
    lam = problem.c - aty
    eq = problem.row_lower == problem.row_upper
    g_rl = np.where(eq, y, np.maximum(y, 0.0))
    g_ru = np.where(eq, 0.0, np.minimum(y, 0.0))
    g_l = np.where(np.isfinite(problem.col_lower), np.maximum(lam, 0.0), 0.0)
    g_u = np.where(np.isfinite(problem.col_upper), np.minimum(lam, 0.0), 0.0)
    return {"c": x.copy(), "row_lower": g_rl, "row_upper": g_ru, "col_lower": g_l, "col_upper": g_u,
            "objective": float(problem.c @ x)}


def _problems(mats: List[SparseMatrix], c, rl, ru, l, u) -> List[Problem]:
    out = []
    for i, A in enumerate(mats):
        out.append(Problem.from_arrays(A, c[i], l[i], u[i], rl[i], ru[i], ObjectiveSense.Minimize, 0.0, f"layer{i}"))
    return out


if torch is not None:

    class LPFunction(torch.autograd.Function):
        """autograd.Function (c, row_lower, row_upper, col_lower, col_upper) -> (x*, v*),
        v* = c^T x* the optimal value of each instance."""

        @staticmethod
        def forward(ctx, c, row_lower, row_upper, col_lower, col_upper, mats, config, adjoint_tol, certify_tol,
                    polish=True):
            host = [t.detach().to("cpu", torch.float64).numpy() for t in (c, row_lower, row_upper, col_lower,
                                                                            col_upper)]
            probs = _problems(mats, *host)
            sols = solve_batch(probs, config)
            for i, s in enumerate(sols):
                if not s.is_optimal():
                    raise RuntimeError(f"LP layer: instance {i} stopped with status {s.status.name}")
            if polish:
                # the vertex of the identified basis: the point the adjoint differentiates
                xp, yp, infos = polish_batch(probs, [s.x for s in sols], [s.row_duals for s in sols],
                                             tolerance=adjoint_tol)
                xs, ys, bad = choose_outputs(sols, xp, yp, infos, certify_tol)
            else:  # the PDHG points as they are (optimal values and their gradients need no basis)
                xs, ys = [s.x for s in sols], [s.row_duals for s in sols]
                infos, bad = None, []
            if bad:
                worst = max(max(infos[i]["primal_violation"], infos[i]["dual_violation"]) for i in bad)
                warnings.warn(f"LP layer: {len(bad)} of {len(probs)} polished bases not optimal (worst relative "
                              f"violation {worst:.2e}); instances {bad[:8]}{'...' if len(bad) > 8 else ''} return "
                              f"their PDHG point and approximate gradients", LPLayerWarning, stacklevel=3)
            ctx.uncertified = bad
            ctx.probs = probs
            ctx.xs, ctx.ys = xs, ys
            ctx.polish_info = infos
            ctx.adjoint_tol = adjoint_tol
            ctx.device = c.device
            ctx.obj_grads = [objective_gradients(p, x, y) for p, x, y in zip(probs, xs, ys)]
            x_t = torch.from_numpy(np.stack(xs)).to(c.device)
            v_t = torch.tensor([d["objective"] for d in ctx.obj_grads], dtype=torch.float64, device=c.device)
            return x_t, v_t

        @staticmethod
        def backward(ctx, grad_x, grad_v):
            keys = ("c", "row_lower", "row_upper", "col_lower", "col_upper")
            out = {k: np.stack([np.zeros_like(d[k]) for d in ctx.obj_grads]) for k in keys}
            if grad_x is not None:
                g = grad_x.detach().to("cpu", torch.float64).numpy()
                if np.any(g):  # the solution map: adjoint system on the identified basis
                    grads, infos = adjoint_batch(ctx.probs, ctx.xs, ctx.ys, list(g), tolerance=ctx.adjoint_tol)
                    ctx.adjoint_info = infos
                    for k in keys:
                        out[k] += np.stack([d[k] for d in grads])
            if grad_v is not None:  # the optimal value: envelope theorem, exact at the returned point
                gv = grad_v.detach().to("cpu", torch.float64).numpy()
                for k in keys:
                    out[k] += gv[:, None] * np.stack([d[k] for d in ctx.obj_grads])
            to_t = lambda k: torch.from_numpy(out[k]).to(ctx.device)
            return (to_t("c"), to_t("row_lower"), to_t("row_upper"), to_t("col_lower"), to_t("col_upper"),
                    None, None, None, None, None)

    def lp_layer(mats: List[SparseMatrix], c, row_lower, row_upper, col_lower, col_upper,
                 config: Optional[GpuPdhgConfig] = None, adjoint_tol: float = 1e-6, certify_tol: float = 1e-6,
                 return_objective: bool = False, polish: bool = True):
        """x* of each LP of the batch (a (batch, n) float64 tensor), differentiable
        with respect to the bounds (and c, with a zero implicit part).  Instances
        whose polished vertex is not certified within ``certify_tol`` return their
        PDHG point (with an LPLayerWarning).  With return_objective, also the
        optimal values v* = c^T x* (a (batch,) tensor) whose gradients come from
        the duals (objective_gradients): write an objective term of a loss as
        v* rather than c^T x* to differentiate it without the basis.  polish=False
        skips the basis polish (the PDHG points are returned as they are): for
        losses of v* alone, whose gradients need no basis, the layer is then one
        batched solve."""
        cfg = config if config is not None else GpuPdhgConfig(max_iterations=1_000_000, tol_primal=1e-6,
                                                               tol_dual=1e-6, tol_gap=1e-6)
        x, v = LPFunction.apply(c, row_lower, row_upper, col_lower, col_upper, list(mats), cfg, adjoint_tol,
                                certify_tol, polish)
        return (x, v) if return_objective else x

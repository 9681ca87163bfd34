"""PyTorch differentiation through batched LP solves.

``solve_lps(c, row_lower, row_upper, col_lower, col_upper, matrices)`` solves B LPs
    min c[k]'x  s.t.  row_lower[k] <= A_k x <= row_upper[k],  col_lower[k] <= x <= col_upper[k]
on the GPU in one batched launch and returns (x*, y*, f*) as float64 tensors of shapes (B, n),
(B, m) and (B,); y* are the row multipliers as SANKHYA reports them (row_dual: the derivative of
f* by a row bound). The PDHG solve stops at `tolerance` (relative KKT, default 1e-7) and is then
polished at its active sets (`polish`, default on), which lands on the vertex for a
nondegenerate optimum. Backpropagation goes through sankhya_gb300_batch_adjoint: the gradients with
respect to c and to the four bound tensors come from implicit differentiation of the optimum
(two basis solves per LP on the device). An equality row passes the same tensor as row_lower and
row_upper; autograd then adds its two halves into dL/db. The matrices are data, not
differentiated: a list of B (col_starts, row_index, values) CSC triples of the same shape (they
may be the same arrays, as for branch-and-bound nodes sharing one A).
"""
from __future__ import annotations

import numpy as np

from . import capi
from .model import LP

try:
    import torch
except ImportError:  # pragma: no cover - torch is optional for the rest of the package
    torch = None


def _rows(t):
    return [np.ascontiguousarray(r, dtype=np.float64) for r in t.detach().cpu().numpy()]


if torch is not None:

    class BatchLPFunction(torch.autograd.Function):
        """Forward: one batched solve. Backward: one batched adjoint."""

        @staticmethod
        def forward(ctx, c, row_lower, row_upper, col_lower, col_upper, matrices, options):
            B, n = c.shape
            m = row_lower.shape[1]
            cs, rls, rus, ls, us = (_rows(t) for t in (c, row_lower, row_upper, col_lower,
                                                       col_upper))
            lps = []
            for k in range(B):
                col_starts, row_index, values = matrices[k]
                lps.append(LP(m, n, col_starts, row_index, values, cs[k], ls[k], us[k], rls[k],
                              rus[k]))
            eng = capi.BatchEngine(options.get("device", 0))
            eng.load(lps)
            items, _ = eng.solve(tolerance=options.get("tolerance", 1e-7),
                                 iteration_limit=options.get("iteration_limit", -1),
                                 stop_rule=options.get("stop_rule", "relative"))
            if options.get("polish", True):
                items, _ = eng.polish()
            xs, ys, fs = [], [], []
            for k, it in enumerate(items):
                if it.status_name not in ("optimal", "feasible"):
                    raise RuntimeError(f"LP {k} of the batch ended {it.status_name}")
                x, _, y = eng.solution(k)
                xs.append(x)
                ys.append(y)
                fs.append(it.objective)
            ctx.engine = eng
            ctx.device = c.device
            dev = c.device
            return (torch.as_tensor(np.stack(xs), device=dev),
                    torch.as_tensor(np.stack(ys), device=dev),
                    torch.as_tensor(np.array(fs), device=dev))

        @staticmethod
        def backward(ctx, gx, gy, gf):
            eng = ctx.engine
            B = gf.shape[0]
            res = eng.adjoint(dl_dx=_rows(gx), dl_dy=_rows(gy),
                              dl_df=gf.detach().cpu().numpy().astype(np.float64))
            bad = [k for k in range(B) if res[k]["status"] != 0]
            if bad:
                raise RuntimeError(f"adjoint failed for LPs {bad[:8]}: "
                                   f"{[res[k]['status'] for k in bad[:8]]}")
            dev = ctx.device

            def stack(key):
                return torch.as_tensor(np.stack([r[key] for r in res]), device=dev)

            return stack("dc"), stack("drl"), stack("dru"), stack("dl"), stack("du"), None, None


def solve_lps(c, row_lower, row_upper, col_lower, col_upper, matrices, **options):
    """Differentiable batched LP solve; see the module docstring."""
    if torch is None:
        raise RuntimeError("PyTorch is not installed")
    return BatchLPFunction.apply(c, row_lower, row_upper, col_lower, col_upper, matrices,
                                 options)

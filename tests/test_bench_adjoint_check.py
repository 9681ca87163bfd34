"""The bench's gradient checks, on the CPU.

`bench.adjoint_section` compares the adjoint's gradients with dense basis solves and with
central finite differences of L = gx.x* + gy.y* + f* over costs, right-hand sides and active
bounds. Here the device engine is replaced by an exact one: every LP (and every perturbed
copy, which shares its matrix arrays) is solved at the planted basis with sparse LU, and the
gradient comes from the same basis. So both checks must agree to rounding, and any slip in the
bench's bookkeeping (which coordinate, which sign, which gradient field) shows up as an error
far above it.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sih-26_gb300"))

sp = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")


class _Item:
    def __init__(self, objective):
        self.objective = objective
        self.iterations = 1
        self.status_name = "optimal"
        self.converged = True


class ExactBatchEngine:
    """BatchEngine's interface, solved exactly at the planted basis of each matrix."""

    bases = {}

    def __init__(self, device):
        self.lps = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def load(self, lps):
        self.lps = list(lps)
        for lp in self.lps:
            if getattr(lp, "x0", None) is not None:
                basic = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
                ExactBatchEngine.bases[id(lp.values)] = (basic, lp.x0 <= lp.col_lower)

    def _parts(self, lp):
        a = sp.csc_matrix((lp.values, lp.row_index, lp.col_starts), shape=(lp.rows, lp.cols))
        basic, at_lower = ExactBatchEngine.bases[id(lp.values)]
        return a, basic, at_lower, spl.splu(a[:, basic].tocsc())

    def _vertex(self, lp):
        a, basic, at_lower, lu = self._parts(lp)
        x = np.where(at_lower, lp.col_lower, lp.col_upper)
        x[basic] = lu.solve(lp.row_lower - a[:, ~basic] @ x[~basic])
        y = lu.solve(lp.col_cost[basic], trans="T")
        return x, y

    def solve(self, **kw):
        self.sol = [self._vertex(lp) for lp in self.lps]
        return [_Item(lp.col_cost @ s[0]) for lp, s in zip(self.lps, self.sol)], 0.0

    def polish(self):
        items, _ = self.solve()
        return items, [{"status": 0} for _ in self.lps]

    def solution(self, k):
        x, y = self.sol[k]
        return x, None, y

    def set_point(self, k, x, d, y):
        """The exact polish below re-solves each LP at its planted basis, so the warm start
        only has to be of the LP's shape."""
        assert x.shape == (self.lps[k].cols,) and y.shape == (self.lps[k].rows,)

    def adjoint(self, gx, gy, gf):
        out = []
        for lp, g_x, g_y in zip(self.lps, gx, gy):
            a, basic, at_lower, lu = self._parts(lp)
            x, y = self._vertex(lp)
            p = lu.solve(g_x[basic], trans="T")
            q = lu.solve(g_y)
            dc = x.copy()
            dc[basic] += q
            dbound = g_x - a.T @ p + (lp.col_cost - a.T @ y)
            out.append({"dc": dc, "drl": p + y, "dru": np.zeros(lp.rows),
                        "dl": np.where(~basic & at_lower, dbound, 0.0),
                        "du": np.where(~basic & ~at_lower, dbound, 0.0),
                        "status": 0, "iterations": [1, 1]})
        return out


def test_adjoint_section_bookkeeping(monkeypatch):
    import bench
    from sankhya_gb300 import build, capi

    build.build_lpgen()
    monkeypatch.setattr(capi, "BatchEngine", ExactBatchEngine)
    out = bench.adjoint_section(0, lps_count=3, shape=(60, 120), ref_lps=2, fd_lps=2,
                                fd_coords=16)
    assert out["max_rel_err_vs_basis_solves"] < 1e-10
    assert set(out["fd_max_rel_err_by_family"]) == {"c", "b", "l", "u"}
    assert out["fd_max_rel_err"] < 1e-5
    assert out["fd_polished"] == 2 * 2 * 16

"""The torch.autograd wrapper (sankhya_gb300.autograd.solve_lps), on the CPU.

The device engine is replaced by an exact one with BatchEngine's interface: each LP is solved
at its planted nondegenerate basis with sparse LU, and its adjoint is the implicit derivative
at that basis. Perturbing c, the row bounds or the active column bounds by a small step keeps
that basis optimal, so the exact forward is affine in each input near the data, and
torch.autograd.gradcheck compares the wrapper's backward with central differences of its own
forward. That checks the wrapper's plumbing: the order of the returned gradients, the batch
stacking, the equality row passed as one tensor for both row bounds (autograd adds the two
halves), and the gradient of f*. The engine's own gradients are checked on the GPU
(tests/test_gpu_adjoint.py).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
sp = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")


class _Item:
    def __init__(self, objective):
        self.objective = objective
        self.status_name = "optimal"


class ExactBatchEngine:
    """sankhya_gb300.capi.BatchEngine's interface, solved exactly at a fixed basis per
    matrix. Rows are equalities at row_lower; row_upper is ignored by the forward, and its
    gradient is zero, as for the engine on an equality row whose lower side is the one
    reported active."""

    bases = {}

    def __init__(self, device=0):
        self.lps = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def load(self, lps):
        self.lps = list(lps)

    def _parts(self, lp):
        a = sp.csc_matrix((lp.values, lp.row_index, lp.col_starts), shape=(lp.rows, lp.cols))
        basic, at_lower = ExactBatchEngine.bases[id(lp.values)]
        return a, basic, at_lower, spl.splu(a[:, basic].tocsc())

    def _vertex(self, lp):
        a, basic, at_lower, lu = self._parts(lp)
        x = np.where(at_lower, lp.col_lower, lp.col_upper)
        x[basic] = lu.solve(lp.row_lower - a[:, ~basic] @ x[~basic])
        return x, lu.solve(lp.col_cost[basic], trans="T")

    def solve(self, **kw):
        self.sol = [self._vertex(lp) for lp in self.lps]
        return [_Item(lp.col_cost @ s[0]) for lp, s in zip(self.lps, self.sol)], 0.0

    def polish(self):
        items, _ = self.solve()
        return items, [{"status": 0} for _ in self.lps]

    def solution(self, k):
        x, y = self.sol[k]
        return x, None, y

    def adjoint(self, dl_dx=None, dl_dy=None, dl_df=None):
        out = []
        for k, lp in enumerate(self.lps):
            a, basic, at_lower, lu = self._parts(lp)
            x, y = self._vertex(lp)
            g_x = np.zeros(lp.cols) if dl_dx is None else dl_dx[k]
            g_y = np.zeros(lp.rows) if dl_dy is None else dl_dy[k]
            g_f = 0.0 if dl_df is None else float(dl_df[k])
            p = lu.solve(g_x[basic], trans="T")
            q = lu.solve(g_y)
            dc = g_f * x
            dc[basic] += q
            dbound = g_x - a.T @ p + g_f * (lp.col_cost - a.T @ y)
            out.append({"dc": dc, "drl": p + g_f * y, "dru": np.zeros(lp.rows),
                        "dl": np.where(~basic & at_lower, dbound, 0.0),
                        "du": np.where(~basic & ~at_lower, dbound, 0.0), "status": 0})
        return out


@pytest.fixture
def planted(monkeypatch, built):
    from sankhya_gb300 import capi, lpgen

    monkeypatch.setattr(capi, "BatchEngine", ExactBatchEngine)
    lps = [lpgen.planted_nondegenerate(12, 24, 4, seed=s) for s in (3, 4)]
    for lp in lps:
        basic = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
        ExactBatchEngine.bases[id(lp.values)] = (basic, lp.x0 <= lp.col_lower)
    return lps


def _inputs(lps):
    def t(key):
        return torch.tensor(np.stack([getattr(lp, key) for lp in lps]), dtype=torch.float64,
                            requires_grad=True)

    return t("col_cost"), t("row_lower"), t("row_upper"), t("col_lower"), t("col_upper")


def test_gradcheck_against_the_wrappers_own_forward(planted):
    from sankhya_gb300.autograd import solve_lps

    mats = [(lp.col_starts, lp.row_index, lp.values) for lp in planted]
    rng = np.random.default_rng(7)
    w = torch.tensor(rng.standard_normal((len(planted), planted[0].cols)))
    v = torch.tensor(rng.standard_normal((len(planted), planted[0].rows)))

    def loss(c, rl, ru, lo, up):
        x, y, f = solve_lps(c, rl, ru, lo, up, mats)
        return (w * x).sum() + (v * y).sum() + f.sum()

    assert torch.autograd.gradcheck(loss, _inputs(planted), eps=1e-6, atol=1e-6, rtol=1e-6)


def test_equality_row_as_one_tensor_and_gradient_of_the_optimum(planted):
    """One tensor b for both row bounds: autograd adds the two halves into dL/db. With
    L = f*, dL/dc = x*, dL/db = y* (the reported row multipliers) and dL/dbound = the reduced
    cost on the nonbasic columns."""
    from sankhya_gb300.autograd import solve_lps

    mats = [(lp.col_starts, lp.row_index, lp.values) for lp in planted]
    c, b, _, lo, up = _inputs(planted)
    x, y, f = solve_lps(c, b, b, lo, up, mats)
    f.sum().backward()
    for k, lp in enumerate(planted):
        assert np.allclose(x[k].detach().numpy(), lp.x0, atol=1e-10)
        assert np.allclose(c.grad[k].numpy(), lp.x0, atol=1e-10)
        assert np.allclose(b.grad[k].numpy(), lp.lam, atol=1e-10)
        d = lp.col_cost - sp.csc_matrix((lp.values, lp.row_index, lp.col_starts),
                                        shape=(lp.rows, lp.cols)).T @ lp.lam
        at_l = lp.x0 <= lp.col_lower
        at_u = lp.x0 >= lp.col_upper
        assert np.allclose(lo.grad[k].numpy(), np.where(at_l, d, 0.0), atol=1e-10)
        assert np.allclose(up.grad[k].numpy(), np.where(at_u, d, 0.0), atol=1e-10)

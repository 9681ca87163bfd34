"""The adjoint (sankhya_gb300_batch_adjoint) against two independent references.

* The basis reference: at the planted nondegenerate optimum the basic columns B are known
  (x0 strictly inside its box), every row is an equality, and the gradients follow from two
  dense solves with A_B (numpy): p = A_B^-T g_x[B], q = A_B^-1 g_y, so
      dL/dc = g_f x* + q on B,  dL/db = p + g_f y*,  dL/dbound_N = g_x[N] - A_N' p + g_f d_N.
* Central finite differences of L through SciPy's HiGHS: re-solving the perturbed LP gives
  the exact vertex, and L is affine in each coordinate near a nondegenerate optimum.

The forward solves stop at relative KKT 1e-7 and are then polished at their active sets
(sankhya_gb300_batch_polish), which must land on the planted vertex. Bar: 1e-5 relative (the
adjoint's accuracy target), measured against max(1, |gradient|).
"""
import numpy as np
import pytest

from sankhya_gb300 import capi, lpgen

pytestmark = pytest.mark.gpu


def dense(lp):
    A = np.zeros((lp.rows, lp.cols))
    for j in range(lp.cols):
        for k in range(lp.col_starts[j], lp.col_starts[j + 1]):
            A[lp.row_index[k], j] = lp.values[k]
    return A


def basis_gradients(lp, gx, gy, gf):
    A = dense(lp)
    x, y = lp.x0, lp.lam
    B = (x > lp.col_lower) & (x < lp.col_upper)
    d = lp.col_cost - A.T @ y
    p = np.linalg.solve(A[:, B].T, gx[B])
    q = np.linalg.solve(A[:, B], gy)
    dc = gf * x.copy()
    dc[B] += q
    db = p + gf * y
    dbound = gx - A.T @ p + gf * d
    dl = np.where(~B & (x <= lp.col_lower), dbound, 0.0)
    du = np.where(~B & (x >= lp.col_upper), dbound, 0.0)
    return dc, db, dl, du


def close(a, b, tol=1e-5):
    return np.all(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b)))


@pytest.mark.parametrize("m", [30, 80, 150])
def test_adjoint_matches_basis_solves(m):
    lps = [lpgen.planted_nondegenerate(m, 2 * m, 5, seed=900 + m + s) for s in range(2)]
    rng = np.random.default_rng(m)
    gxs = [rng.standard_normal(lp.cols) for lp in lps]
    gys = [rng.standard_normal(lp.rows) for lp in lps]
    gfs = np.ones(len(lps))
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        items, _ = eng.solve(tolerance=1e-7, stop_rule="relative", iteration_limit=1000000)
        assert all(it.status_name in ("optimal", "feasible") for it in items)
        polished, info = eng.polish()
        assert all(i["status"] == 0 for i in info), info
        assert all(it.status_name == "optimal" for it in polished)
        for k, lp in enumerate(lps):
            x, _, y = eng.solution(k)
            assert np.allclose(x, lp.x0, rtol=0, atol=1e-9)
            assert np.allclose(y, lp.lam, rtol=0, atol=1e-9)
        res = eng.adjoint(gxs, gys, gfs)
    for lp, gx, gy, r in zip(lps, gxs, gys, res):
        assert r["status"] == 0, r
        assert r["basic_cols"] == lp.rows == r["active_rows"]
        dc, db, dl, du = basis_gradients(lp, gx, gy, 1.0)
        assert close(r["dc"], dc)
        assert close(r["drl"] + r["dru"], db)
        assert close(r["dl"], dl) and close(r["du"], du)


def test_adjoint_matches_finite_differences_through_highs():
    so = pytest.importorskip("scipy.optimize")
    sp = pytest.importorskip("scipy.sparse")
    lp = lpgen.planted_nondegenerate(40, 80, 5, seed=77)
    A = sp.csc_matrix((lp.values, lp.row_index, lp.col_starts), shape=(lp.rows, lp.cols))
    rng = np.random.default_rng(5)
    gx, gy = rng.standard_normal(lp.cols), rng.standard_normal(lp.rows)

    def loss(c, b, lo, up):
        h = so.linprog(c, A_eq=A, b_eq=b, bounds=list(zip(lo, up)), method="highs")
        assert h.status == 0
        return gx @ h.x + gy @ h.eqlin.marginals + h.fun

    with capi.BatchEngine(0) as eng:
        eng.load([lp])
        eng.solve(tolerance=1e-7, stop_rule="relative", iteration_limit=1000000)
        eng.polish()
        r = eng.adjoint([gx], [gy], [1.0])[0]
    assert r["status"] == 0
    h = 1e-5
    basic = np.flatnonzero((lp.x0 > 0) & (lp.x0 < 10))
    upper = np.flatnonzero(lp.x0 >= 10)
    lower = np.flatnonzero(lp.x0 <= 0)
    checks = [("c", j) for j in rng.choice(lp.cols, 6, replace=False)]
    checks += [("b", i) for i in rng.choice(lp.rows, 4, replace=False)]
    checks += [("u", j) for j in upper[:3]] + [("l", j) for j in lower[:3]]
    for kind, k in checks:
        args = [lp.col_cost.copy(), lp.row_lower.copy(), lp.col_lower.copy(), lp.col_upper.copy()]
        idx = {"c": 0, "b": 1, "l": 2, "u": 3}[kind]
        plus = [a.copy() for a in args]
        minus = [a.copy() for a in args]
        plus[idx][k] += h
        minus[idx][k] -= h
        fd = (loss(*plus) - loss(*minus)) / (2 * h)
        if kind == "b":
            got = r["drl"][k] + r["dru"][k]
        else:
            got = r[{"c": "dc", "l": "dl", "u": "du"}[kind]][k]
        assert abs(got - fd) <= 1e-5 * max(1.0, abs(fd)), (kind, k, got, fd)
    assert len(basic) == lp.rows


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from sankhya_gb300.autograd import solve_lps

    lps = [lpgen.planted_nondegenerate(25, 50, 5, seed=s) for s in (1, 2)]
    mats = [(lp.col_starts, lp.row_index, lp.values) for lp in lps]
    c = torch.tensor(np.stack([lp.col_cost for lp in lps]), requires_grad=True)
    b = torch.tensor(np.stack([lp.row_lower for lp in lps]), requires_grad=True)
    lo = torch.tensor(np.stack([lp.col_lower for lp in lps]), requires_grad=True)
    up = torch.tensor(np.stack([lp.col_upper for lp in lps]), requires_grad=True)
    x, y, f = solve_lps(c, b, b, lo, up, mats, tolerance=1e-7, iteration_limit=1000000)
    rng = np.random.default_rng(0)
    w = torch.tensor(rng.standard_normal(x.shape))
    v = torch.tensor(rng.standard_normal(y.shape))
    L = (w * x).sum() + (v * y).sum() + f.sum()
    L.backward()
    for k, lp in enumerate(lps):
        assert np.allclose(x[k].detach().numpy(), lp.x0, atol=1e-9)
        dc, db, dl, du = basis_gradients(lp, w[k].numpy(), v[k].numpy(), 1.0)
        assert close(c.grad[k].numpy(), dc)
        assert close(b.grad[k].numpy(), db)
        assert close(lo.grad[k].numpy(), dl) and close(up.grad[k].numpy(), du)


def test_adjoint_of_a_maximisation_lp():
    """max (-c)'x over the planted LP's feasible set has the same optimum x*; its reported
    row duals are -y* and its objective -f*. With L' = w'x* + v'y' + f' the chain rule gives
    dL'/dc' = -(the minimisation's dL/dc for upstream w, -v, -1), and every other gradient
    equal to the minimisation's for that upstream."""
    from sankhya_gb300.model import LP

    lp = lpgen.planted_nondegenerate(60, 120, 5, seed=4242)
    mx = LP(lp.rows, lp.cols, lp.col_starts, lp.row_index, lp.values, -lp.col_cost,
            lp.col_lower, lp.col_upper, lp.row_lower, lp.row_upper, sense=-1.0)
    rng = np.random.default_rng(11)
    w, v = rng.standard_normal(lp.cols), rng.standard_normal(lp.rows)
    with capi.BatchEngine(0) as eng:
        eng.load([mx])
        items, _ = eng.solve(tolerance=1e-7, stop_rule="relative", iteration_limit=1000000)
        assert items[0].status_name in ("optimal", "feasible")
        _, info = eng.polish()
        assert info[0]["status"] == 0, info
        x, _, y = eng.solution(0)
        assert np.allclose(x, lp.x0, rtol=0, atol=1e-9)
        assert np.allclose(y, -lp.lam, rtol=0, atol=1e-9)
        r = eng.adjoint([w], [v], [1.0])[0]
    assert r["status"] == 0, r
    dc, db, dl, du = basis_gradients(lp, w, -v, -1.0)
    assert close(r["dc"], -dc)
    assert close(r["drl"] + r["dru"], db)
    assert close(r["dl"], dl) and close(r["du"], du)


def test_polish_from_a_set_point_matches_the_adjoint_at_step_1e6():
    """Perturbed copies of a planted LP (costs and right-hand sides moved by +-1e-6) are
    solved, then polished from the base LP's vertex (sankhya_gb300_batch_set_point): each
    lands on its own vertex (the dense solve at the planted basis), and the central
    differences of L = g_x'x* + g_y'y* + f* match the adjoint to 1e-5 relative."""
    from sankhya_gb300.model import LP

    lp = lpgen.planted_nondegenerate(80, 160, 5, seed=31)
    rng = np.random.default_rng(8)
    gx, gy = rng.standard_normal(lp.cols), rng.standard_normal(lp.rows)
    h = 1e-6
    with capi.BatchEngine(0) as eng:
        eng.load([lp])
        eng.solve(tolerance=1e-7, stop_rule="relative", iteration_limit=1000000)
        eng.polish()
        base = eng.solution(0)
        r = eng.adjoint([gx], [gy], [1.0])[0]
    assert r["status"] == 0, r
    picks = [("c", int(j)) for j in rng.choice(lp.cols, 4, replace=False)]
    picks += [("b", int(i)) for i in rng.choice(lp.rows, 4, replace=False)]
    pert = []
    for fam, j in picks:
        for sign in (1.0, -1.0):
            c, rl = lp.col_cost.copy(), lp.row_lower.copy()
            if fam == "c":
                c[j] += sign * h
            else:
                rl[j] += sign * h
            pert.append(LP(lp.rows, lp.cols, lp.col_starts, lp.row_index, lp.values, c,
                           lp.col_lower, lp.col_upper, rl, rl.copy()))
    A = dense(lp)
    B = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
    with capi.BatchEngine(0) as eng:
        eng.load(pert)
        eng.solve(tolerance=1e-4, stop_rule="relative", iteration_limit=1000000)
        for q in range(len(pert)):
            eng.set_point(q, *base)
        _, info = eng.polish()
        assert all(i["status"] == 0 for i in info), info
        sols = [eng.solution(q) for q in range(len(pert))]
    for q, p in enumerate(pert):
        x = np.where(lp.x0 <= lp.col_lower, lp.col_lower, lp.col_upper)
        x[B] = np.linalg.solve(A[:, B], p.row_lower - A[:, ~B] @ x[~B])
        assert np.allclose(sols[q][0], x, rtol=0, atol=1e-10), q
    for t, (fam, j) in enumerate(picks):
        (xp, _, yp), (xm, _, ym) = sols[2 * t], sols[2 * t + 1]
        dl = (gx + lp.col_cost) @ (xp - xm) + gy @ (yp - ym)
        if fam == "c":
            dl += h * (xp[j] + xm[j])
        fd = dl / (2 * h)
        got = r["dc"][j] if fam == "c" else r["drl"][j] + r["dru"][j]
        assert abs(got - fd) <= 1e-5 * max(1.0, abs(fd)), (fam, j, got, fd)


def test_polish_leaves_degenerate_and_infeasible_lps_alone():
    degenerate = lpgen.planted_uniform(40, 80, 5, seed=3)  # more interior columns than rows
    with capi.BatchEngine(0) as eng:
        eng.load([degenerate])
        items, _ = eng.solve(tolerance=1e-8, iteration_limit=400000)
        x_before = eng.solution(0)[0]
        polished, info = eng.polish()
        assert info[0]["status"] == 1
        assert polished[0].status_name == items[0].status_name
        assert np.array_equal(eng.solution(0)[0], x_before)

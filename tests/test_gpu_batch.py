"""The batched engine (one thread block per LP, one persistent launch) against the oracle.

Each LP of a batch must come out as the reference's PDHG would solve it alone: the same
status, the objective within 1e-6 relative of the oracle's, and the reported point's
relative KKT (re-evaluated by the oracle's evaluate) within the tolerance. LPs sharing a
matrix (branch-and-bound node relaxations) are checked against SciPy's HiGHS for status and
objective; infeasible ones must be reported infeasible.
"""
import numpy as np
import pytest

from sankhya_gb300 import capi, certify, lpgen
from sankhya_gb300.model import LP, from_dense

pytestmark = pytest.mark.gpu
INF = np.inf


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def _mixed_batch():
    lps = [lpgen.planted_uniform(m, 2 * m, 5, seed=100 + m) for m in (30, 57, 120, 200, 333)]
    lps += [lpgen.planted_general(40, 60, 3, seed=200 + s, maximize=s == 1, free=False)
            for s in range(3)]
    lps.append(lpgen.planted_blocks(4, 50, 100, 9, seed=5))
    lps.append(from_dense([[1, 1]], [2], [INF], [1, 1]))
    lps.append(from_dense([[1, 0], [0, 2], [3, 2]], [-INF] * 3, [4, 12, 18], [3, 5], sense=-1))
    return lps


def test_batch_matches_oracle(oracle):
    lps = _mixed_batch()
    tol = 1e-8
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        items, seconds = eng.solve(tolerance=tol, iteration_limit=400000)
        for k, (lp, it) in enumerate(zip(lps, items)):
            ref = oracle.solve(lp, tolerance=tol, iteration_limit=400000)
            print(f"{k}: {it.status_name} {it.iterations} it vs oracle {ref.status_name} "
                  f"{ref.iterations} it; obj {it.objective!r} vs {ref.objective!r}")
            assert it.status_name == ref.status_name
            assert rel(it.objective, ref.objective) <= 1e-6
            x, d, y = eng.solution(k)
            res, _, red = oracle.evaluate(lp, x, -lp.sense * y)
            assert max(res["primal"], res["dual"], res["gap"]) <= tol, (k, res)
            assert np.allclose(lp.sense * red, d, rtol=1e-12, atol=1e-12)
    assert seconds > 0.0


def test_batch_stop_at_request_and_relative_rule(oracle):
    lps = [lpgen.planted_uniform(m, 2 * m, 5, seed=7 + m) for m in (40, 90)]
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        items, _ = eng.solve(tolerance=1e-6, stop_rule="relative")
        for k, it in enumerate(items):
            assert it.status_name in ("optimal", "feasible")
            res = it.residuals
            assert max(res["primal"], res["dual"], res["gap"]) <= 1e-6
        items, _ = eng.solve(tolerance=1e-6, stop_at_request=True)
        for it in items:
            assert it.status_name in ("optimal", "feasible")


def test_batch_iteration_limit_and_reproducible():
    lps = [lpgen.planted_uniform(m, 2 * m, 5, seed=m) for m in (60, 80, 100)]
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        eng.set_schedule(2, 256)  # a fixed schedule: bit-reproducible solves
        a, _ = eng.solve(tolerance=1e-12, iteration_limit=321)
        assert all(it.status_name == "iteration_limit" and it.iterations == 321 for it in a)
        b, _ = eng.solve(tolerance=1e-12, iteration_limit=321)
        for p, q in zip(a, b):
            assert p.objective == q.objective and p.attempts == q.attempts
        xa = eng.solution(1)[0]
        eng.solve(tolerance=1e-12, iteration_limit=321)
        assert np.array_equal(xa, eng.solution(1)[0])


def _node(base, rng, tighten):
    """A branch-and-bound style relaxation of `base`: `tighten` variables' bounds tightened
    to [0, floor(x0_j)] or [ceil(x0_j), 10]; the matrix arrays are SHARED with `base`."""
    l = base.col_lower.copy()
    u = base.col_upper.copy()
    for j in rng.choice(base.cols, size=tighten, replace=False):
        if rng.random() < 0.5:
            u[j] = np.floor(base.x0[j])
        else:
            l[j] = np.ceil(base.x0[j])
    return LP(base.rows, base.cols, base.col_starts, base.row_index, base.values,
              base.col_cost, l, u, base.row_lower, base.row_upper)


def test_batch_nodes_share_one_matrix_against_highs():
    scipy_opt = pytest.importorskip("scipy.optimize")
    from scipy.sparse import csc_matrix

    base = lpgen.planted_uniform(60, 120, 5, seed=11)
    rng = np.random.default_rng(3)
    nodes = [_node(base, rng, int(t)) for t in rng.integers(1, 21, size=24)]
    # Some nodes infeasible for sure: every column fixed at 0 cannot meet A x = b != 0.
    for k in range(0, 24, 6):
        zero = np.zeros(base.cols)
        nodes[k] = LP(base.rows, base.cols, base.col_starts, base.row_index, base.values,
                      base.col_cost, zero, zero.copy(), base.row_lower, base.row_upper)
    A = csc_matrix((base.values, base.row_index, base.col_starts), shape=(base.rows, base.cols))
    eng = capi.BatchEngine(0)
    eng.load(nodes)
    items, _ = eng.solve(tolerance=1e-8, iteration_limit=200000)
    for k, (lp, it) in enumerate(zip(nodes, items)):
        h = scipy_opt.linprog(lp.col_cost, A_eq=A, b_eq=lp.row_lower,
                              bounds=list(zip(lp.col_lower, lp.col_upper)), method="highs")
        print(k, it.status_name, it.iterations, it.objective, "highs", h.status,
              h.fun if h.status == 0 else None)
        if h.status == 2:
            assert it.status_name == "infeasible", (k, it)
            assert it.farkas_value > 0.0
            # The certificate itself, checked on the host in exactly rounded FP64.
            assert certify.farkas_share(lp, eng.ray(k)) > 0.0, k
        else:
            assert h.status == 0
            assert it.status_name in ("optimal", "feasible"), (k, it)
            assert rel(it.objective, h.fun) <= 1e-6
    eng.close()


def test_batch_reports_infeasible_lps():
    bad = [from_dense([[1, 1]], [5], [5], [1, 1], col_upper=[1, 1]),           # x1 + x2 = 5
           from_dense([[1, -1], [1, 1]], [3, -INF], [INF, 1], [1, 2],           # x1 - x2 >= 3,
                      col_upper=[2, 2])]                                        # x1 + x2 <= 1
    good = [from_dense([[1, 1]], [1], [1], [1, 2], col_upper=[1, 1])]
    with capi.BatchEngine(0) as eng:
        eng.load(bad + good)
        items, _ = eng.solve(tolerance=1e-8, iteration_limit=100000)
        rays = [eng.ray(k) for k in range(2)]
    assert [it.status_name for it in items[:2]] == ["infeasible", "infeasible"]
    assert items[2].status_name == "optimal" and rel(items[2].objective, 1.0) <= 1e-6
    for lp, d in zip(bad, rays):
        assert certify.farkas_share(lp, d) > 0.0


def test_batch_rejects_bad_lps():
    lp = lpgen.planted_uniform(20, 40, 5, seed=1)
    bad = LP(lp.rows, lp.cols, lp.col_starts, lp.row_index, lp.values, lp.col_cost,
             lp.col_upper, lp.col_lower, lp.row_lower, lp.row_upper)  # l > u
    with capi.BatchEngine(0) as eng:
        with pytest.raises(capi.EngineError):
            eng.load([lp, bad])
        eng.load([lp])
        items, _ = eng.solve(tolerance=1e-6)
        assert items[0].status_name in ("optimal", "feasible")


@pytest.mark.parametrize("rule", ["relative", "standard"])
def test_batch_mixed_precision_matches_oracle(oracle, rule):
    """The mixed method per LP (FP32 iterations on FP64 refinement rounds) reaches the
    requested relative KKT on the FP64 evaluation, with the oracle's objective."""
    lps = _mixed_batch()
    tol = 1e-8
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        items, _ = eng.solve(tolerance=tol, iteration_limit=400000, precision="mixed",
                             stop_rule=rule)
        for k, (lp, it) in enumerate(zip(lps, items)):
            ref = oracle.solve(lp, tolerance=tol, iteration_limit=400000)
            print(f"{k}: {it.status_name} {it.iterations} it {it.refinements} rounds; obj "
                  f"{it.objective!r} vs {ref.objective!r}")
            assert it.status_name in ("optimal", "feasible"), (k, it)
            if rule == "standard":
                assert it.status_name == "optimal", (k, it)
            assert rel(it.objective, ref.objective) <= 1e-6
            x, d, y = eng.solution(k)
            res, _, red = oracle.evaluate(lp, x, -lp.sense * y)
            assert max(res["primal"], res["dual"], res["gap"]) <= tol, (k, res)


def test_batch_mixed_reports_infeasible_lps():
    bad = [from_dense([[1, 1]], [5], [5], [1, 1], col_upper=[1, 1])]
    good = [lpgen.planted_uniform(50, 100, 5, seed=8)]
    with capi.BatchEngine(0) as eng:
        eng.load(bad + good)
        items, _ = eng.solve(tolerance=1e-6, iteration_limit=200000, precision="mixed",
                             stop_rule="relative")
        ray = eng.ray(0)
    assert items[0].status_name == "infeasible"
    assert certify.farkas_share(bad[0], ray) > 0.0
    assert items[1].status_name in ("optimal", "feasible")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_every_schedule_gives_the_same_answers(oracle, precision):
    """Each fixed schedule (lanes per row or column x threads per LP) solves the batch to the
    tolerance with the oracle's statuses and objectives; the autotuned solve reports the
    schedule it picked, which is one of the candidates."""
    lps = _mixed_batch()
    tol = 1e-8
    refs = [oracle.solve(lp, tolerance=tol, iteration_limit=400000) for lp in lps]
    with capi.BatchEngine(0) as eng:
        eng.load(lps)
        for lanes, threads in [(1, 128), (2, 512), (4, 256), (8, 128), (16, 256), (32, 512)]:
            eng.set_schedule(lanes, threads)
            items, _ = eng.solve(tolerance=tol, iteration_limit=400000, precision=precision,
                                 stop_rule="relative")
            assert eng.last_schedule()[:2] == (lanes, threads)
            for k, (lp, it, ref) in enumerate(zip(lps, items, refs)):
                assert it.status_name in ("optimal", "feasible"), (lanes, threads, k, it)
                assert rel(it.objective, ref.objective) <= 1e-6, (lanes, threads, k)
                x, _, y = eng.solution(k)
                res, _, _ = oracle.evaluate(lp, x, -lp.sense * y)
                assert max(res["primal"], res["dual"], res["gap"]) <= tol, (lanes, threads, k)
        eng.set_schedule(0, 0)
        items, _ = eng.solve(tolerance=tol, iteration_limit=400000, precision=precision,
                             stop_rule="relative")
        lanes, threads, tune_s = eng.last_schedule()
        assert lanes in (1, 2, 4, 8) and threads in (128, 256, 512) and tune_s > 0.0
        assert all(rel(it.objective, ref.objective) <= 1e-6 for it, ref in zip(items, refs))
        for bad in [(3, 256), (2, 100), (0, 256), (64, 512)]:
            with pytest.raises(capi.EngineError):
                eng.set_schedule(*bad)

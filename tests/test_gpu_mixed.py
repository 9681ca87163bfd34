"""The mixed-precision method (FP32 PDHG + FP64 refinement rounds) against the oracle.

Same bar as the FP64 engine: the returned point, re-evaluated by the oracle's copy of the
reference's evaluate(), meets the requested relative KKT tolerance; the objective agrees with
the oracle's FP64 PDHG (and the planted optimum) to 1e-6 relative; the status is the one the
reference's rules give that point.
"""
import numpy as np
import pytest

from sankhya_gb300 import capi, lpgen
from sankhya_gb300.model import from_dense

pytestmark = pytest.mark.gpu
INF = np.inf


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def _cases():
    yield "uniform_200x500", lpgen.planted_uniform(200, 500, 5, seed=3)
    yield "uniform_2000x5000", lpgen.planted_uniform(2000, 5000, 5, seed=1)
    yield "blocks", lpgen.planted_blocks(8, 100, 200, 9, seed=4)
    for s in range(3):
        yield f"general_{s}", lpgen.planted_general(40, 60, 3, seed=200 + s, maximize=s == 1,
                                                    free=False)
    yield "range_row", from_dense([[1]], [2], [6], [1])
    yield "maximise", from_dense([[1, 0], [0, 2], [3, 2]], [-INF] * 3, [4, 12, 18], [3, 5],
                                 sense=-1)


@pytest.mark.parametrize("rule", ["relative", "standard"])
@pytest.mark.parametrize("name,lp", list(_cases()), ids=[c[0] for c in _cases()])
def test_mixed_matches_oracle(engine, oracle, name, lp, rule):
    tol = 1e-8
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": tol, "pdhg_precision": "mixed",
                                   "pdhg_stop_rule": rule, "iteration_limit": 400000},
                              engine=engine)
    ref = oracle.solve(lp, tolerance=tol, iteration_limit=400000)
    r = sol.result
    print(f"{name}/{rule}: {sol.status} {sol.iterations} it, {r.refinements} rounds, obj "
          f"{sol.objective!r} vs oracle {ref.objective!r} ({ref.status_name}), "
          f"rel {rel(sol.objective, ref.objective):.2e}")
    assert sol.status in ("optimal", "feasible"), sol.message
    if rule == "standard":
        assert sol.status == "optimal"
    assert rel(sol.objective, ref.objective) <= 1e-6
    if lp.fstar is not None and lp.sense > 0:
        assert rel(sol.objective, lp.fstar) <= 1e-6
    res, _, red = oracle.evaluate(lp, sol.col_value, -lp.sense * sol.row_dual)
    assert max(res["primal"], res["dual"], res["gap"]) <= tol, res
    assert np.allclose(lp.sense * red, sol.col_dual, rtol=1e-12, atol=1e-12)
    # The engine reports the reference's residuals of its point (FP64, unscaled).
    for key in ("primal", "dual", "gap"):
        assert abs(r.residuals[key] - res[key]) <= 1e-12 + 1e-6 * res[key]


def test_mixed_iteration_limit(engine):
    lp = lpgen.planted_uniform(300, 700, 5, seed=5)
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-12, "pdhg_precision": "mixed",
                                   "iteration_limit": 100}, engine=engine)
    assert sol.status == "iteration_limit"
    assert sol.iterations <= 100
    assert np.isinf(sol.dual_bound)


def test_mixed_is_bit_reproducible(engine):
    lp = lpgen.planted_uniform(300, 700, 5, seed=6)
    opts = {"pdhg_tolerance": 1e-8, "pdhg_precision": "mixed"}
    a = capi.solve_pdhg_gpu(lp, opts, engine=engine)
    b = capi.solve_pdhg_gpu(lp, opts, engine=engine)
    assert a.iterations == b.iterations and a.objective == b.objective
    assert np.array_equal(a.col_value, b.col_value)

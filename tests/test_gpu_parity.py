"""GPU engine against the oracle, through the C ABI.

Bars (see each test):
* device preconditioning: Dr, Dc and the scaled values bit-identical to the reference's
  build_scaling; the spectral-norm estimate within 1e-14 relative (its two norms are summed
  in a different order);
* sparse products: SparseMatrix::multiply / transpose_multiply's summation order, with
  FMA, so every entry is within 1e-14 * sum |a_ij| |v_j| of the reference's (a few ulps), on
  short rows and on long rows summed in chunks;
* solves: the same status, the objective within 1e-6 relative of the oracle's (the
  engine's parity bar; the achieved difference is printed), the reported point's relative KKT
  (re-evaluated by the oracle's own evaluate) within the requested tolerance.
"""
import numpy as np
import pytest

from sankhya_gb300 import capi, lpgen
from sankhya_gb300.model import LP, from_dense

pytestmark = pytest.mark.gpu
INF = np.inf
OBJ_TOL = 1e-6  # relative objective agreement with the oracle (the engine's parity bar)


def rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def test_scaling_bit_identical(engine, oracle):
    lp = lpgen.planted_blocks(6, 50, 100, 9, seed=21)
    engine.load(lp)
    dr, dc, vals, norm = engine.scaling(random_seed=0)
    ref = oracle.build_scaling(lp)
    assert np.array_equal(dr, ref["row"])
    assert np.array_equal(dc, ref["col"])
    assert np.array_equal(vals, ref["values"])
    ref_lp = LP(lp.rows, lp.cols, lp.col_starts, lp.row_index, ref["values"], lp.col_cost,
                lp.col_lower, lp.col_upper, lp.row_lower, lp.row_upper)
    ref_norm = oracle.spectral_norm(ref_lp, 30, 1)
    assert rel(norm, ref_norm) <= 1e-14, (norm, ref_norm)


def _abs_product(lp, v, transpose):
    """(|A| |v|)_i: the scale of the rounding error of a sum of products."""
    a = LP(lp.rows, lp.cols, lp.col_starts, lp.row_index, np.abs(lp.values), lp.col_cost,
           lp.col_lower, lp.col_upper, lp.row_lower, lp.row_upper)
    return a, np.abs(v)


def assert_spmv_close(oracle, lp, got, v, transpose):
    want = oracle.transpose_multiply(lp, v) if transpose else oracle.multiply(lp, v)
    a, av = _abs_product(lp, v, transpose)
    scale = oracle.transpose_multiply(a, av) if transpose else oracle.multiply(a, av)
    # The engine accumulates with FMA in the reference's order; each product-and-add then
    # rounds once instead of twice, so the bound is a few ulps of sum |a_ij| |v_j|.
    assert np.all(np.abs(got - want) <= 1e-14 * scale + 1e-300), np.max(np.abs(got - want) / scale)


def test_spmv_matches_reference_products(engine, oracle):
    lp = lpgen.planted_general(300, 500, 4, seed=5)
    engine.load(lp)
    rng = np.random.default_rng(1)
    x = rng.normal(size=lp.cols)
    x[::7] = 0.0
    y = rng.normal(size=lp.rows)
    assert_spmv_close(oracle, lp, engine.spmv(0, x), x, False)
    assert_spmv_close(oracle, lp, engine.spmv(1, y), y, True)


def _long_row_lp(m=40, n=6000, seed=2):
    """Row 0 is dense (n nonzeros > one tile); the rest are sparse."""
    rng = np.random.default_rng(seed)
    starts, rows, vals = [0], [], []
    for j in range(n):
        r = sorted({0} | set(rng.integers(1, m, size=2).tolist()))
        rows += r
        vals += rng.normal(size=len(r)).tolist()
        starts.append(len(rows))
    return LP(m, n, np.array(starts, np.int32), np.array(rows, np.int32), np.array(vals),
              np.zeros(n), np.zeros(n), np.full(n, 10.0), np.zeros(m), np.zeros(m))


def test_spmv_long_rows(engine, oracle):
    lp = _long_row_lp()
    engine.load(lp)
    rng = np.random.default_rng(3)
    x = rng.normal(size=lp.cols)
    assert_spmv_close(oracle, lp, engine.spmv(0, x), x, False)  # row 0 is 3 chunks long
    y = rng.normal(size=lp.rows)
    assert_spmv_close(oracle, lp, engine.spmv(1, y), y, True)


def _solve_cases():
    yield "sum", from_dense([[1, 1]], [2], [INF], [1, 1]), dict(tolerance=1e-8), 2.0
    yield "equality", from_dense([[1, 1]], [4], [4], [1, 2]), dict(tolerance=1e-8), 4.0
    yield "range_row", from_dense([[1]], [2], [6], [1]), dict(tolerance=1e-8), 2.0
    yield ("col_upper", from_dense([[1]], [-INF], [100], [-1], col_upper=[7]),
           dict(tolerance=1e-8), -7.0)
    yield ("maximise", from_dense([[1, 0], [0, 2], [3, 2]], [-INF] * 3, [4, 12, 18], [3, 5],
                                  sense=-1), dict(tolerance=1e-8), 36.0)
    yield ("offset", from_dense([[1]], [3], [INF], [1], offset=10.0), dict(tolerance=1e-8), 13.0)
    yield "big_rhs", from_dense([[1, 1]], [1e5], [INF], [1, 1]), dict(tolerance=1e-4), 1e5
    yield "uniform_200x500", lpgen.planted_uniform(200, 500, 5, seed=3), dict(tolerance=1e-8), None
    yield ("uniform_2000x5000", lpgen.planted_uniform(2000, 5000, 5, seed=1),
           dict(tolerance=1e-8), None)
    yield "blocks", lpgen.planted_blocks(8, 100, 200, 9, seed=4), dict(tolerance=1e-8), None
    for s in range(4):
        yield (f"general_{s}", lpgen.planted_general(30, 45, 3, seed=100 + s, maximize=s % 2 == 1,
                                                     free=False),
               dict(tolerance=1e-6, iteration_limit=100000), None)
    yield ("stop_at_request", lpgen.planted_uniform(100, 250, 5, seed=9),
           dict(tolerance=1e-6, stop_at_request=True), None)
    yield ("no_restarts", lpgen.planted_uniform(100, 250, 5, seed=9),
           dict(tolerance=1e-8, restart=False, iteration_limit=3000), None)


@pytest.mark.parametrize("name,lp,kw,exact", list(_solve_cases()),
                         ids=[c[0] for c in _solve_cases()])
def test_solve_matches_oracle(engine, oracle, name, lp, kw, exact):
    ref = oracle.solve(lp, **kw)
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": kw["tolerance"],
                                   "iteration_limit": kw.get("iteration_limit", -1),
                                   "pdhg_restart": kw.get("restart", True),
                                   "pdhg_stop_at_request": kw.get("stop_at_request", False)},
                              engine=engine)
    print(f"{name}: gpu {sol.status} {sol.iterations} it obj {sol.objective!r}; "
          f"oracle {ref.status_name} {ref.iterations} it obj {ref.objective!r}; "
          f"rel {rel(sol.objective, ref.objective):.2e}")
    if kw.get("stop_at_request"):
        # With pdhg_stop_at_request the loop stops on the request and the status is
        # `optimal` only if that point happens to meet the project standard too
        # (src/pdhg/pdhg.cpp:416-423): where two trajectories stop decides it, so either
        # verdict is the reference's behaviour as long as the request itself was met.
        assert sol.status in ("optimal", "feasible") and ref.status_name in ("optimal",
                                                                            "feasible")
    else:
        assert sol.status == ref.status_name, sol.message
    if sol.status in ("optimal", "feasible"):
        assert rel(sol.objective, ref.objective) <= OBJ_TOL
        if exact is not None:
            assert abs(sol.objective - exact) <= 1e-6 * max(1.0, abs(exact))
        if lp.fstar is not None and lp.sense > 0:
            assert rel(sol.objective, lp.fstar) <= OBJ_TOL
        # The oracle's own evaluate of the reported point (the reference's residuals).
        r, _, red = oracle.evaluate(lp, sol.col_value, -lp.sense * sol.row_dual)
        tol = kw["tolerance"]
        assert r["primal"] <= tol and r["dual"] <= tol and r["gap"] <= tol, r
        assert r["absolute_primal"] <= 1e-7
        assert np.allclose(lp.sense * red, sol.col_dual, rtol=1e-12, atol=1e-12)
    if sol.status == "optimal":
        assert np.isfinite(sol.dual_bound)
        assert rel(sol.dual_bound, sol.objective) <= 1e-6
    else:
        assert np.isinf(sol.dual_bound)


@pytest.mark.parametrize("seed", [100, 102])
def test_free_rows_and_columns_converge_in_kkt(engine, oracle, seed):
    """With free rows / columns the status depends on whether a multiplier rounds to exactly
    zero (see lpgen.c); what must hold is that the relative KKT reaches the request."""
    lp = lpgen.planted_general(30, 45, 3, seed=seed, free=True)
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-6, "iteration_limit": 30000},
                              engine=engine)
    r, _, _ = oracle.evaluate(lp, sol.col_value, -lp.sense * sol.row_dual)
    assert max(r["primal"], r["dual"], r["gap"]) <= 1e-6, r
    assert rel(sol.objective, lp.fstar) <= 1e-5


def test_iteration_limit_is_exact(engine, oracle):
    lp = from_dense([[1, 1]], [2], [INF], [1, 1])
    for limit in (0, 1, 20, 41):
        sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-12, "iteration_limit": limit},
                                  engine=engine)
        ref = oracle.solve(lp, tolerance=1e-12, iteration_limit=limit)
        assert sol.status == ref.status_name == "iteration_limit"
        assert sol.iterations == ref.iterations == limit
        assert np.isinf(sol.dual_bound) and sol.message


def test_runs_are_bit_reproducible(engine):
    lp = lpgen.planted_uniform(300, 800, 5, seed=12)
    a = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-8}, engine=engine)
    b = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-8}, engine=engine)
    assert a.iterations == b.iterations and a.objective == b.objective
    assert np.array_equal(a.col_value, b.col_value) and np.array_equal(a.row_dual, b.row_dual)


def test_model_error_is_a_status(engine):
    lp = lpgen.planted_uniform(20, 40, 3, seed=1)
    lp.values = lp.values.copy()
    lp.values[5] = np.nan
    sol = capi.solve_pdhg_gpu(lp, {}, engine=engine)
    assert sol.status == "model_error"


def test_zero_time_limit(engine):
    lp = lpgen.planted_uniform(50, 100, 3, seed=1)
    sol = capi.solve_pdhg_gpu(lp, {"time_limit": 0.0}, engine=engine)
    assert sol.status == "time_limit" and sol.iterations == 0


def test_interrupt_flag_stops_the_loop(engine):
    lp = lpgen.planted_uniform(500, 1200, 5, seed=2)
    flag = np.ones(1, dtype=np.int32)  # already raised: stops at the first poll
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-12, "steps_per_poll": 8},
                              engine=engine, interrupt=flag)
    assert sol.status == "interrupted"
    assert 0 < sol.iterations <= 64


def test_iteration_log_every_40(engine):
    lp = lpgen.planted_uniform(200, 500, 5, seed=3)
    rows = []
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": 1e-8}, engine=engine,
                              log=lambda it, obj, p, d, s: rows.append((it, obj, p, d)))
    assert sol.status == "optimal"
    assert rows and all(it % 40 == 0 for it, *_ in rows[:-1])
    assert abs(rows[-1][1] - sol.objective) <= 1e-6 * max(1.0, abs(sol.objective))


def test_engines_on_two_devices_in_one_process(oracle):
    """Each device gets its own kernel configuration (the shared-memory opt-ins are per
    device): engines on devices 0 and 1 in one process each run a product and a solve. It
    uses no peer memory. Skips where fewer than two GPUs are visible."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("fewer than two GPUs are visible")
    lp = lpgen.planted_uniform(200, 500, 5, seed=3)
    x = np.random.default_rng(4).normal(size=lp.cols)
    ref = oracle.solve(lp, tolerance=1e-8)
    for device in (0, 1):
        with capi.PdhgEngine(device) as eng:
            eng.load(lp)
            assert_spmv_close(oracle, lp, eng.spmv(0, x), x, False)
            r = eng.solve(tolerance=1e-8)
            assert r.status_name == ref.status_name
            assert rel(r.objective, ref.objective) <= OBJ_TOL

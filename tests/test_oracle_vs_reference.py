"""The oracle (oracle/pdhg_oracle.c) against the reference's own PDHG, compiled from its
sources into oracle/_ref/, on identical inputs: every result must be bit-identical
(src/pdhg/pdhg.cpp, src/la/scaling.cpp, src/pdhg/pdhg_evaluate.cpp)."""
import numpy as np
import pytest

from sankhya_gb300 import lpgen
from sankhya_gb300.model import from_dense

INF = np.inf


def _cases():
    yield "uniform_200x500", lpgen.planted_uniform(200, 500, 5, seed=3), dict(tolerance=1e-8)
    for s in range(3):
        yield (f"general_{s}", lpgen.planted_general(40, 60, 3, seed=s, maximize=s == 1,
                                                     free=s != 2),
               dict(tolerance=1e-8, iteration_limit=20000))
    yield "sum", from_dense([[1, 1]], [2], [INF], [1, 1]), dict(tolerance=1e-8)
    yield ("max_3x2", from_dense([[1, 0], [0, 2], [3, 2]], [-INF] * 3, [4, 12, 18], [3, 5],
                                 sense=-1), dict(tolerance=1e-8))
    yield "big_rhs", from_dense([[1, 1]], [1e5], [INF], [1, 1]), dict(tolerance=1e-4)
    yield ("iteration_limit", from_dense([[1, 1]], [2], [INF], [1, 1]),
           dict(tolerance=1e-12, iteration_limit=20))
    yield ("stop_at_request", lpgen.planted_uniform(100, 250, 5, seed=9),
           dict(tolerance=1e-6, stop_at_request=True))
    yield ("no_restarts", lpgen.planted_uniform(100, 250, 5, seed=9),
           dict(tolerance=1e-8, restart=False, iteration_limit=3000))
    yield ("seed_5", lpgen.planted_uniform(100, 250, 5, seed=9),
           dict(tolerance=1e-6, random_seed=5))
    # Zipf row lengths and values of log-uniform magnitude over [1e-3, 1e3]: the badly scaled
    # family, where the scaling does the most work.
    yield ("zipf_badly_scaled", lpgen.planted_zipf(300, 600, 6000, max_len=400, seed=4),
           dict(tolerance=1e-8, iteration_limit=20000))


@pytest.mark.parametrize("name,lp,kw", list(_cases()), ids=[c[0] for c in _cases()])
def test_solve_is_bit_identical(reference, oracle, name, lp, kw):
    a = oracle.solve(lp, **kw)
    b = reference.solve(lp, **kw)
    assert a.status == b.status, (a.status_name, b.status_name, b.message)
    assert a.iterations == b.iterations
    if b.restarts >= 0:  # the feasible-status message carries no restart count
        assert a.restarts == b.restarts
    assert a.objective == b.objective
    assert a.dual_bound == b.dual_bound or (np.isinf(a.dual_bound) and np.isinf(b.dual_bound))
    assert np.array_equal(a.col_value, b.col_value)
    assert np.array_equal(a.col_dual, b.col_dual)
    assert np.array_equal(a.row_dual, b.row_dual)


_SCALING_CASES = [
    ("blocks", lambda: lpgen.planted_blocks(4, 60, 120, 9, seed=11)),
    ("zipf_badly_scaled", lambda: lpgen.planted_zipf(300, 600, 6000, max_len=400, seed=4)),
    ("general_free", lambda: lpgen.planted_general(50, 80, 3, seed=6, maximize=True, free=True)),
]


@pytest.mark.parametrize("make", [c[1] for c in _SCALING_CASES], ids=[c[0] for c in _SCALING_CASES])
def test_scaling_and_norm_are_bit_identical(reference, oracle, make):
    lp = make()
    a = oracle.build_scaling(lp)
    b = reference.build_scaling(lp)
    for k in ("values", "row", "col", "cost", "col_lower", "col_upper", "row_lower", "row_upper",
              "min_abs", "max_abs"):
        assert np.array_equal(a[k], b[k]), k
    assert oracle.spectral_norm(lp, 30, 1) == reference.spectral_norm(lp, 30, 1)


@pytest.mark.parametrize("make", [c[1] for c in _SCALING_CASES], ids=[c[0] for c in _SCALING_CASES])
def test_evaluate_is_bit_identical(reference, oracle, make):
    lp = make()
    rng = np.random.default_rng(0)
    x = rng.normal(size=lp.cols)
    y = rng.normal(size=lp.rows)
    ra, aa, da = oracle.evaluate(lp, x, y)
    rb, ab, db = reference.evaluate(lp, x, y)
    assert ra == rb
    assert np.array_equal(aa, ab) and np.array_equal(da, db)


def test_inputs_at_the_edge_of_validation(reference, oracle):
    """Model::validate (src/core/model.cpp:214,228) refuses a NaN objective offset and lets an
    infinite cost through. A NaN offset is a model error on both. With +inf on a column
    bounded below, the projection holds the column at its bound: both run to the iteration
    limit with a NaN objective, bit for bit alike. (With the cost pushing a column towards an
    infinite bound the reference never ends, so that case is not run; the engine refuses any
    infinite cost.)"""
    nan_offset = from_dense([[1, 1]], [2], [INF], [1, 1], offset=float("nan"))
    for impl in (oracle, reference):
        assert impl.solve(nan_offset, tolerance=1e-8).status_name == "model_error"
    lp = from_dense([[1, 1]], [2], [INF], [INF, 1.0], col_upper=[10, 10])
    a = oracle.solve(lp, tolerance=1e-8, iteration_limit=400)
    b = reference.solve(lp, tolerance=1e-8, iteration_limit=400)
    assert a.status_name == b.status_name == "iteration_limit"
    assert a.iterations == b.iterations == 400 and a.restarts == b.restarts
    assert np.isnan(a.objective) and np.isnan(b.objective)
    for u, v in ((a.col_value, b.col_value), (a.col_dual, b.col_dual), (a.row_dual, b.row_dual)):
        assert np.array_equal(u, v, equal_nan=True)


def _random_lp(rng, m, n, density):
    """A random m x n matrix in CSC with the given density (explicit zeros dropped)."""
    dense = np.where(rng.random((m, n)) < density, rng.normal(size=(m, n)), 0.0)
    starts, rows, vals = [0], [], []
    for j in range(n):
        nz = np.flatnonzero(dense[:, j])
        rows += nz.tolist()
        vals += dense[nz, j].tolist()
        starts.append(len(rows))
    from sankhya_gb300.model import LP

    lp = LP(m, n, np.array(starts, np.int32), np.array(rows, np.int32), np.array(vals),
            np.zeros(n), np.zeros(n), np.full(n, 1.0), np.zeros(m), np.zeros(m))
    return lp, dense


def test_products_match_the_reference_and_a_dense_product(reference, oracle):
    """The oracle's A x and A^T y (src/la/sparse.cpp:232-269) against the reference's own
    SparseMatrix products, bit for bit, and against a dense product to 1e-9 as the
    reference's FuzzMatVecAgainstDenseReference holds them (tests/unit/test_sparse.cpp:190-226):
    500 matrices of 1-40 rows and columns at densities 0.02, 0.1, 0.4 and 0.95. A third of the
    vector entries are zero (A x skips those columns) and some are -0.0."""
    rng = np.random.default_rng(20260825)
    densities = (0.02, 0.1, 0.4, 0.95)
    for trial in range(500):
        m, n = (int(v) for v in rng.integers(1, 41, size=2))
        lp, dense = _random_lp(rng, m, n, densities[trial % 4])
        x = rng.normal(size=n)
        x[rng.random(n) < 1 / 3] = 0.0
        x[rng.random(n) < 0.05] = -0.0
        y = rng.normal(size=m)
        ax, aty = oracle.multiply(lp, x), oracle.transpose_multiply(lp, y)
        assert np.array_equal(ax, reference.multiply(lp, x)), trial
        assert np.array_equal(np.signbit(ax), np.signbit(reference.multiply(lp, x))), trial
        assert np.array_equal(aty, reference.transpose_multiply(lp, y)), trial
        assert np.all(np.abs(ax - dense @ x) <= 1e-9), trial
        assert np.all(np.abs(aty - dense.T @ y) <= 1e-9), trial

"""The GPU convex-QP engine (sankhya_gb300_qp_*) against the oracle's restatement of the
reference's solve_convex_qp (oracle/qp_oracle.c, pinned bit for bit to the reference by
tests/test_qp_oracle.py).

Bars: the same status and iteration count as the oracle (the trajectories differ only in the
rounding of the FMA-accumulated sums, a few ulps per product); the point, the duals and the
objective within 1e-9 relative of the oracle's scale; bit-identical answers from repeated
solves; the reference's hand-derived optima (tests/unit/test_qp.cpp); the limits, the
interrupt and the log as the reference applies them.
"""
import json
import os

import numpy as np
import pytest

from sankhya_gb300 import capi
from sankhya_gb300.model import LP, QP, qp_from_dense, random_qp

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_qp.json")) as f:
    GOLDEN = json.load(f)["cases"]
INF = float("inf")
TOL = 1e-9  # relative to the vector's scale


@pytest.fixture(scope="module")
def qp_engine(built):
    eng = capi.QpEngine(0)
    yield eng
    eng.close()


def decode(d):
    from test_qp_oracle import decode as dec

    return dec(d)


def close(a, b, tol=TOL):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    return a.shape == b.shape and (a.size == 0 or float(np.max(np.abs(a - b))) <= tol * scale)


def solve_both(qp_engine, oracle, qp, **options):
    qp_engine.load(qp)
    r = qp_engine.solve(**options)
    x, d, y = qp_engine.solution()
    o = oracle.solve_qp(qp, **{k: v for k, v in options.items()
                               if k in ("tolerance", "iteration_limit", "time_limit",
                                        "random_seed")})
    return r, (x, d, y), o


def assert_same(r, got, o, tol=TOL):
    x, d, y = got
    assert r.status_name == o.status_name, r.message
    assert r.iterations == o.iterations, r.message
    assert close(x, o.col_value, tol), np.max(np.abs(x - o.col_value))
    assert close(d, o.col_dual, tol), np.max(np.abs(d - o.col_dual))
    assert close(y, o.row_dual, tol), np.max(np.abs(y - o.row_dual))
    assert abs(r.objective - o.objective) <= tol * max(1.0, abs(o.objective))


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_qp_matches_oracle_on_golden(qp_engine, oracle, case):
    qp = decode(case["qp"])
    r, got, o = solve_both(qp_engine, oracle, qp, **case["options"])
    assert o.iterations == case["iterations"]  # the oracle is the reference here
    assert_same(r, got, o)
    assert abs(r.norm_a - o.norm_a) <= 1e-12 * max(1.0, o.norm_a)
    assert abs(r.norm_q - o.norm_q) <= 1e-12 * max(1.0, o.norm_q)


KNOWN = [
    (lambda: qp_from_dense([-2.0, -8.0], [0, 0], [INF, INF], [(0, 0, 2.0), (1, 1, 4.0)]),
     [1.0, 2.0], -9.0, 1e-6),
    (lambda: qp_from_dense([-2.0, -8.0], [0, 0], [0.25, INF], [(0, 0, 2.0), (1, 1, 4.0)]),
     [0.25, 2.0], -8.4375, 1e-6),
    (lambda: qp_from_dense([0.0, 0.0], [0, 0], [INF, INF], [(0, 0, 1.0), (1, 1, 1.0)],
                           [[1.0, 1.0]], [2.0], [2.0]), [1.0, 1.0], 1.0, 1e-5),
    (lambda: qp_from_dense([-4.0, -4.0], [0, 0], [INF, INF],
                           [(0, 0, 2.0), (1, 0, 1.0), (1, 1, 2.0)]),
     [4.0 / 3.0, 4.0 / 3.0], -16.0 / 3.0, 1e-5),
    (lambda: qp_from_dense([2.0], [0], [INF], [(0, 0, -1.0)], sense=-1.0), [2.0], 2.0, 1e-5),
]


@pytest.mark.parametrize("k", range(len(KNOWN)))
def test_qp_known_answers(qp_engine, k):
    """tests/unit/test_qp.cpp's hand-derived optima."""
    make, x, f, tol = KNOWN[k]
    qp_engine.load(make())
    r = qp_engine.solve(tolerance=1e-10, iteration_limit=500000)
    assert r.status_name == "optimal", r.message
    got = qp_engine.solution()[0]
    assert np.allclose(got, x, atol=tol, rtol=0)
    assert abs(r.objective - f) <= tol


def long_items_qp(seed=5, m=3000, n=2500):
    """A QP with rows and columns long enough for the chunked path at every lane count: two
    dense rows, one column in every row, and a Hessian row that couples 2,600 columns."""
    base = random_qp(seed, m, n, per_column=3, hessian_band=1)
    a = base.lp
    rng = np.random.default_rng(seed)
    starts, index, values = [0], [], []
    for j in range(n):
        rows = set(a.row_index[a.col_starts[j]:a.col_starts[j + 1]].tolist()) | {0, 1}
        if j == 7:
            rows = set(range(m))
        rows = sorted(rows)
        index.extend(rows)
        values.extend(rng.normal(size=len(rows)).tolist())
        starts.append(len(index))
    starts = np.array(starts, np.int32)
    index = np.array(index, np.int32)
    values = np.array(values)
    x0 = np.clip(rng.uniform(-1, 1, size=n), a.col_lower, a.col_upper)
    ax = np.zeros(m)
    for j in range(n):
        ax[index[starts[j]:starts[j + 1]]] += values[starts[j]:starts[j + 1]] * x0[j]
    rl, ru = ax - 1.0, ax + 1.0
    lp = LP(m, n, starts, index, values, a.col_cost, a.col_lower, a.col_upper, rl, ru)
    # Hessian: the base band and diagonal, plus column 3 coupled to every other column.
    hs, hi, hv = base.hessian_starts, base.hessian_index, base.hessian_values
    triples = []
    for j in range(n):
        for k in range(hs[j], hs[j + 1]):
            triples.append((int(hi[k]), j, float(hv[k])))
    extra = {}
    for i in range(4, n):
        extra[(i, 3)] = 1e-3 * rng.normal()
    diag_boost = sum(abs(v) for v in extra.values())
    triples = [(i, j, v + (diag_boost if i == j == 3 else 0.0) + (1e-3 if i == j else 0.0))
               for i, j, v in triples if (i, j) not in extra] + [(i, j, v) for (i, j), v in extra.items()]
    from sankhya_gb300.model import hessian_from_triples

    hs, hi, hv = hessian_from_triples(n, triples)
    return QP(lp, hs, hi, hv, "long_items")


@pytest.mark.parametrize("lanes", [(1, 1), (4, 8), (32, 32), (0, 0)])
def test_qp_long_items_every_lane_count(qp_engine, oracle, lanes):
    qp = long_items_qp()
    r, got, o = solve_both(qp_engine, oracle, qp, tolerance=1e-6, iteration_limit=3000,
                           column_lanes=lanes[0], row_lanes=lanes[1])
    if lanes != (0, 0):
        assert (r.column_lanes, r.row_lanes) == lanes
    assert_same(r, got, o, tol=1e-8)


@pytest.mark.parametrize("make,options", [
    (lambda: random_qp(41, 300, 600), dict(tolerance=1e-8)),
    (lambda: random_qp(42, 500, 800, maximise=True, per_column=5), dict(tolerance=1e-7)),
    (lambda: random_qp(43, 0, 400), dict(tolerance=1e-10)),
    (lambda: QP(random_qp(44, 200, 400).lp, np.zeros(401, np.int32), np.zeros(0, np.int32),
                np.zeros(0)), dict(tolerance=1e-6, iteration_limit=5000)),
    (lambda: random_qp(45, 200, 400), dict(tolerance=1e-8, iteration_limit=1237)),
    (lambda: random_qp(46, 200, 400), dict(tolerance=1e-8, random_seed=99)),
], ids=["min", "max", "no_rows", "no_hessian", "cut_odd", "seed"])
def test_qp_matches_oracle(qp_engine, oracle, make, options):
    qp = make()
    r, got, o = solve_both(qp_engine, oracle, qp, **options)
    assert_same(r, got, o)


def test_qp_reproducible(qp_engine):
    qp_engine.load(random_qp(51, 400, 700))
    a = qp_engine.solve(tolerance=1e-8)
    xa = qp_engine.solution()
    b = qp_engine.solve(tolerance=1e-8)
    xb = qp_engine.solution()
    assert a.iterations == b.iterations and a.objective == b.objective
    for u, v in zip(xa, xb):
        assert np.array_equal(u, v)


def test_qp_limits_interrupt_and_log(qp_engine, oracle):
    # Tolerance 1e-30 is never met (the residuals stop near rounding level), so every run
    # below ends at a limit, an interrupt or the log's last line.
    qp = random_qp(52, 200, 400)
    qp_engine.load(qp)
    r = qp_engine.solve(tolerance=1e-30, iteration_limit=0)
    assert r.status_name == "iteration_limit" and r.iterations == 0
    r = qp_engine.solve(tolerance=1e-8, time_limit=0.0)
    assert r.status_name == "time_limit" and r.iterations == 0
    x, _, _ = qp_engine.solution()
    assert np.array_equal(x, np.clip(0.0, qp.lp.col_lower, qp.lp.col_upper))
    flag = np.ones(1, np.int32)
    r = qp_engine.solve(tolerance=1e-30, interrupt=flag, periods_per_poll=2)
    assert r.status_name == "interrupted" and r.iterations == 100
    calls = []
    r = qp_engine.solve(tolerance=1e-30, poll=lambda it, obj: calls.append(it) or len(calls) >= 3,
                        periods_per_poll=1)
    assert r.status_name == "interrupted" and calls == [50, 100, 150] and r.iterations == 150
    logged = []
    r = qp_engine.solve(tolerance=1e-30, iteration_limit=10000,
                        log=lambda it, obj, p, d, s: logged.append((it, obj, p, d)))
    assert r.status_name == "iteration_limit" and r.iterations == 10000
    assert [e[0] for e in logged] == [5000, 10000]
    o = oracle.solve_qp(qp, tolerance=1e-30, iteration_limit=10000)
    assert abs(logged[-1][1] - o.objective) <= 1e-9 * max(1.0, abs(o.objective))
    assert abs(logged[-1][2] - o.primal_residual) <= 1e-9 * max(1e-12, o.primal_residual) + 1e-15
    assert abs(logged[-1][3] - o.dual_residual) <= 1e-9 * max(1e-12, o.dual_residual) + 1e-15
    assert r.kernel_launches > 20000


@pytest.mark.parametrize("hessian,fragment", [
    ([(0, 0, 1.0), (1, 1, -1.0)], "not convex"),
    ([(0, 0, 1.0), (5, 1, 1.0)], "out of range"),
    ([(0, 0, float("nan"))], "not finite"),
])
def test_qp_load_refusals(qp_engine, hessian, fragment):
    from sankhya_gb300.model import hessian_from_triples

    lp = qp_from_dense([0.0, 0.0], [-INF, -INF], [INF, INF], []).lp
    hs, hi, hv = hessian_from_triples(2, [t for t in hessian if t[0] < 2])
    if fragment == "out of range":
        hs = np.array([0, 1, 2], np.int32)
        hi = np.array([0, 5], np.int32)
        hv = np.array([1.0, 1.0])
    with pytest.raises(capi.EngineError) as e:
        qp_engine.load(QP(lp, hs, hi, hv))
    assert e.value.code == 3 and fragment in str(e.value)


def test_qp_time_kernels_keeps_the_answer(qp_engine):
    qp_engine.load(random_qp(53, 300, 600))
    qp_engine.solve(tolerance=1e-8)
    before = qp_engine.solution()
    col, row = qp_engine.time_kernels(5)
    assert col > 0.0 and row > 0.0
    after = qp_engine.solution()
    for u, v in zip(before, after):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("name", ["qp_blend.mps", "crude_blend_qp.mps"])
def test_qp_reference_demo_models(qp_engine, oracle, reference, name):
    """The reference's demo QPs read by its own reader (on the GPU machine from the staged
    copy); qp_blend's optimum is LN = 200/3, HN = 100/3, objective 200/3."""
    import pyoracle

    path = os.path.join(pyoracle.reference_tree(), "demo", name)
    if not os.path.exists(path):
        pytest.skip(f"{name} is not staged")
    qp = reference.read_qp(path)
    r, got, o = solve_both(qp_engine, oracle, qp, tolerance=1e-8)
    assert_same(r, got, o)
    if name == "qp_blend.mps":
        assert np.allclose(got[0], [200.0 / 3.0, 100.0 / 3.0], rtol=1e-6)


@pytest.mark.parametrize("make", [lambda: random_qp(61, 3000, 5000, per_column=6),
                                  lambda: long_items_qp(7)], ids=["random", "long_items"])
def test_qp_staging_gives_the_same_bits(qp_engine, make):
    """The one-lane passes stage each warp's matrix slice in shared memory; the sums are the
    same, in the same order, as reading the matrix directly."""
    qp_engine.load(make())
    a = qp_engine.solve(tolerance=1e-8, iteration_limit=3000, column_lanes=1, row_lanes=1,
                        staging=True)
    xa = qp_engine.solution()
    b = qp_engine.solve(tolerance=1e-8, iteration_limit=3000, column_lanes=1, row_lanes=1)
    xb = qp_engine.solution()
    assert (a.status_name, a.iterations, a.objective) == (b.status_name, b.iterations,
                                                          b.objective)
    for u, v in zip(xa, xb):
        assert np.array_equal(u, v)


def test_qp_python_mirror_on_the_gpu(built, oracle):
    """sankhya_gb300.capi.solve_convex_qp_gpu on the real engine: the oracle's status,
    iteration count and point, the bound only when optimal, a model error for a negative
    diagonal."""
    qp = random_qp(91, 200, 400)
    s = capi.solve_convex_qp_gpu(qp, {"qp_tolerance": 1e-8})
    o = oracle.solve_qp(qp, tolerance=1e-8)
    assert (s.status, s.iterations) == (o.status_name, o.iterations)
    assert close(s.col_value, o.col_value) and close(s.row_dual, o.row_dual)
    assert s.status == "optimal" and s.dual_bound == s.objective
    bad = qp_from_dense([0.0, 0.0], [-INF, -INF], [INF, INF], [(0, 0, 1.0), (1, 1, -1.0)])
    assert capi.solve_convex_qp_gpu(bad).status == "model_error"

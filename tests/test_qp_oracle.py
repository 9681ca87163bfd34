"""The convex-QP oracle (oracle/qp_oracle.c) pinned to the reference's own QP engine.

* Golden: the committed outputs of the reference's solve_convex_qp
  (tests/golden/reference_qp.json, made by tests/golden/make_golden_qp.py) reproduced bit for
  bit: status, iterations, objective and the three vectors. The restatement uses only IEEE
  basic operations and sqrt with no fused multiply-add, so this holds on x86-64 and aarch64.
* Known answers: the hand-derived optima of the reference's tests/unit/test_qp.cpp.
* Side by side with the reference's build (where the reference tree is present): more QPs,
  limits, and the reference's convexity refusals and demo QPs.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from sankhya_gb300.model import LP, QP, qp_from_dense, random_qp

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_qp.json")) as f:
    GOLDEN = json.load(f)["cases"]
INF = float("inf")


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def decode(d):
    def f(key):
        return np.array([float.fromhex(v) for v in d[key]], dtype=np.float64)

    def i(key):
        return np.array(d[key], dtype=np.int32)

    lp = LP(d["rows"], d["cols"], i("col_starts"), i("row_index"), f("values"), f("col_cost"),
            f("col_lower"), f("col_upper"), f("row_lower"), f("row_upper"), sense=d["sense"],
            objective_offset=float.fromhex(d["objective_offset"]))
    return QP(lp, i("hessian_starts"), i("hessian_index"), f("hessian_values"))


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_oracle_reproduces_reference_qp(built, oracle, case):
    qp = decode(case["qp"])
    s = oracle.solve_qp(qp, **case["options"])
    assert s.status_name == case["status"]
    assert s.iterations == case["iterations"]
    assert float(s.objective).hex() == case["objective"]
    assert digest(s.col_value) == case["col_value_sha256"]
    assert digest(s.col_dual) == case["col_dual_sha256"]
    assert digest(s.row_dual) == case["row_dual_sha256"]


# tests/unit/test_qp.cpp: (builder, expected x, expected objective, tolerance).
KNOWN = {
    "separable": (lambda: qp_from_dense([-2.0, -8.0], [0, 0], [INF, INF],
                                        [(0, 0, 2.0), (1, 1, 4.0)]), [1.0, 2.0], -9.0, 1e-6),
    "bound_cuts_off": (lambda: qp_from_dense([-2.0, -8.0], [0, 0], [0.25, INF],
                                             [(0, 0, 2.0), (1, 1, 4.0)]),
                       [0.25, 2.0], -8.4375, 1e-6),
    "coupling_row": (lambda: qp_from_dense([0.0, 0.0], [0, 0], [INF, INF],
                                           [(0, 0, 1.0), (1, 1, 1.0)], [[1.0, 1.0]], [2.0],
                                           [2.0]), [1.0, 1.0], 1.0, 1e-5),
    "off_diagonal_twice": (lambda: qp_from_dense([-4.0, -4.0], [0, 0], [INF, INF],
                                                 [(0, 0, 2.0), (1, 0, 1.0), (1, 1, 2.0)]),
                           [4.0 / 3.0, 4.0 / 3.0], None, 1e-5),
    "maximisation": (lambda: qp_from_dense([2.0], [0], [INF], [(0, 0, -1.0)], sense=-1.0),
                     [2.0], 2.0, 1e-5),
}


@pytest.mark.parametrize("name", sorted(KNOWN))
def test_oracle_known_answers(built, oracle, name):
    make, x, f, tol = KNOWN[name]
    qp = make()
    s = oracle.solve_qp(qp, tolerance=1e-10, iteration_limit=500000)
    assert s.status_name == "optimal"
    assert np.allclose(s.col_value, x, atol=tol, rtol=0)
    want = qp.objective(np.array(x)) if f is None else f
    assert abs(s.objective - want) <= tol


def test_oracle_singular_semidefinite(built, oracle):
    # Q = [[1, 1], [1, 1]]: optimal wherever x + y = 2, value -2 (test_qp.cpp:178-190).
    qp = qp_from_dense([-2.0, -2.0], [0, 0], [10.0, 10.0], [(0, 0, 1.0), (1, 0, 1.0), (1, 1, 1.0)])
    s = oracle.solve_qp(qp, tolerance=1e-9, iteration_limit=500000)
    assert s.status_name == "optimal"
    assert abs(s.col_value.sum() - 2.0) <= 1e-4 and abs(s.objective + 2.0) <= 1e-4


def test_oracle_reported_point(built, oracle):
    """The Solution's duals as src/qp/qp_condat_vu.cpp:343-353 fill them: col_dual = c + Qx +
    sense A'y with y = -sense row_dual; at the optimum of a minimisation whose bounds are not
    active the reduced costs vanish."""
    qp = qp_from_dense([0.0, 0.0], [0, 0], [INF, INF], [(0, 0, 1.0), (1, 1, 1.0)], [[1.0, 1.0]],
                       [2.0], [2.0])
    s = oracle.solve_qp(qp, tolerance=1e-10, iteration_limit=500000)
    q = qp.hessian_dense()
    a = qp.lp.to_dense()
    y = -qp.lp.sense * s.row_dual
    d = qp.lp.col_cost + q @ s.col_value + qp.lp.sense * (a.T @ y)
    assert np.allclose(s.col_dual, d, atol=1e-14, rtol=1e-12)
    assert np.allclose(s.col_dual, 0.0, atol=1e-8)
    assert abs(s.row_dual[0] - 1.0) <= 1e-6  # lambda = 1 (test_qp.cpp:96-98)


def test_oracle_norms(built, oracle):
    qp = random_qp(21, 40, 70)
    na, nq = oracle.qp_norms(qp)
    sa = np.linalg.norm(qp.lp.to_dense(), 2)
    sq = np.abs(np.linalg.eigvalsh(qp.hessian_dense())).max()
    assert 0.9 * sa <= na <= sa * (1 + 1e-12)
    assert 0.9 * sq <= nq <= sq * (1 + 1e-12)


def test_oracle_limits(built, oracle):
    qp = random_qp(22, 30, 60)
    s = oracle.solve_qp(qp, tolerance=1e-14, iteration_limit=123)
    assert s.status_name == "iteration_limit" and s.iterations == 123
    s = oracle.solve_qp(qp, tolerance=1e-8, time_limit=0.0)
    assert s.status_name == "time_limit" and s.iterations == 0
    s = oracle.solve_qp(qp, tolerance=1e-8, iteration_limit=0)
    assert s.status_name == "iteration_limit" and s.iterations == 0


# ---- Side by side with the reference's own build -----------------------------------------

@pytest.mark.parametrize("make,options", [
    (lambda: random_qp(31, 60, 120), dict(tolerance=1e-8)),
    (lambda: random_qp(32, 80, 100, maximise=True, per_column=3), dict(tolerance=1e-7)),
    (lambda: random_qp(33, 20, 40, hessian_band=0), dict(tolerance=1e-9)),
    (lambda: QP(random_qp(34, 30, 60).lp, np.zeros(61, np.int32), np.zeros(0, np.int32),
                np.zeros(0)), dict(tolerance=1e-6, iteration_limit=4000)),
    (lambda: random_qp(35, 30, 60), dict(tolerance=1e-8, iteration_limit=999)),
    (lambda: random_qp(36, 30, 60), dict(tolerance=1e-8, time_limit=0.0)),
], ids=["min", "max", "diagonal", "no_hessian", "cut", "time0"])
def test_oracle_matches_reference_build(built, oracle, reference, make, options):
    qp = make()
    a = oracle.solve_qp(qp, **options)
    b = reference.solve_qp(qp, **options)
    assert (a.status_name, a.iterations) == (b.status_name, b.iterations), b.message
    assert float(a.objective).hex() == float(b.objective).hex()
    for k in ("col_value", "col_dual", "row_dual"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("name,triples", [
    ("negative_curvature", [(0, 0, 1.0), (1, 1, -1.0)]),
    ("hidden_off_diagonal", [(0, 0, 1.0), (1, 0, 3.0), (1, 1, 1.0)]),
])
def test_reference_refuses_nonconvex(reference, name, triples):
    """test_qp.cpp:147-176: the reference refuses these before any arithmetic; its convexity
    test is what the GPU seam runs before the engine."""
    qp = qp_from_dense([0.0, 0.0], [-INF, -INF], [INF, INF], triples)
    s = reference.solve_qp(qp, tolerance=1e-10, iteration_limit=500000)
    assert s.status_name == "model_error" and "not convex" in s.message
    verdict, detail = reference.check_convexity(qp)
    assert verdict == 1 and detail


@pytest.mark.parametrize("name", ["qp_blend.mps", "crude_blend_qp.mps"])
def test_reference_demo_qps(built, oracle, reference, name):
    """The reference's two demo QPs read by its own reader and solved by both; qp_blend's
    optimum is LN = 200/3, HN = 100/3, objective 200/3 (its header derives it)."""
    import pyoracle

    tree = pyoracle.reference_tree()
    path = os.path.join(tree, "demo", name)
    if not os.path.exists(path):
        pytest.skip(f"{name} is not in the reference tree or its staged copy")
    qp = reference.read_qp(path)
    a = oracle.solve_qp(qp, tolerance=1e-8)
    b = reference.solve_qp(qp, tolerance=1e-8)
    assert (a.status_name, a.iterations) == (b.status_name, b.iterations) == ("optimal",
                                                                              b.iterations)
    assert np.array_equal(a.col_value, b.col_value)
    if name == "qp_blend.mps":
        assert np.allclose(a.col_value, [200.0 / 3.0, 100.0 / 3.0], rtol=1e-6)
        assert abs(a.objective - 200.0 / 3.0) <= 1e-5


@pytest.mark.parametrize("seed", range(100, 124))
def test_oracle_matches_reference_build_on_random_qps(built, oracle, reference, seed):
    """Twenty-four more seeded convex QPs of varied shape, density, band and sense: the
    restatement and the reference's own build agree bit for bit."""
    rng = np.random.default_rng(seed)
    m = int(rng.integers(0, 60))
    n = int(rng.integers(5, 90))
    qp = random_qp(seed, m, n, per_column=int(rng.integers(1, 6)),
                   hessian_band=int(rng.integers(0, 4)), maximise=bool(seed % 2))
    options = dict(tolerance=float(10.0 ** -rng.integers(6, 10)), iteration_limit=20000,
                   random_seed=int(rng.integers(0, 5)))
    a = oracle.solve_qp(qp, **options)
    b = reference.solve_qp(qp, **options)
    assert (a.status_name, a.iterations) == (b.status_name, b.iterations), b.message
    assert float(a.objective).hex() == float(b.objective).hex()
    for k in ("col_value", "col_dual", "row_dual"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k

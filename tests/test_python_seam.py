"""The Python mirror of the seam (sankhya_gb300.capi.solve_pdhg_gpu), on the CPU.

Every GPU test drives the engine through this function, so its option plumbing is checked
here without a GPU: the engine is replaced by a stand-in with PdhgEngine's interface that
hands the LP to the oracle (the CPU restatement of the reference PDHG, pinned bit for bit to
it). With the registry's option names set away from their defaults, and with none set, the
mirror must return exactly what the oracle returns for the same settings, and the registry's
defaults (src/util/options.cpp: pdhg_tolerance 1e-4, iteration_limit -1, no time limit,
restarts on, stop_at_request off, random_seed 0) must reach the engine. A model defect is the
status "model_error", as the reference's seam reports it.
"""
import numpy as np
import pytest

from sankhya_gb300 import capi, lpgen
from sankhya_gb300.model import from_dense

INF = np.inf


class _Result:
    def __init__(self, s):
        self.status_name = s.status_name
        self.objective = s.objective
        self.dual_bound = s.dual_bound
        self.iterations = s.iterations
        self.message = s.message


class OracleEngine:
    """PdhgEngine's interface over the oracle. Records the settings each solve received."""

    def __init__(self, oracle):
        self.oracle = oracle
        self.lp = None
        self.calls = []

    def load(self, lp):
        problem = lp.validate()
        if not problem and not all(np.all(np.isfinite(a)) for a in (lp.values, lp.col_cost)):
            problem = "a matrix value or a cost is not finite"
        if problem:
            raise capi.EngineError(3, problem)
        self.lp = lp

    def solve(self, tolerance, iteration_limit, time_limit, restart, stop_at_request,
              random_seed, precision, steps_per_poll, interrupt, log, stop_rule):
        self.calls.append(dict(tolerance=tolerance, iteration_limit=iteration_limit,
                               time_limit=time_limit, restart=restart,
                               stop_at_request=stop_at_request, random_seed=random_seed,
                               precision=precision, stop_rule=stop_rule))
        assert precision == "fp64" and stop_rule == "standard", "the oracle runs the reference"
        self.sol = self.oracle.solve(self.lp, tolerance=tolerance,
                                     iteration_limit=iteration_limit, time_limit=time_limit,
                                     restart=restart, stop_at_request=stop_at_request,
                                     random_seed=random_seed)
        return _Result(self.sol)

    def solution(self):
        return self.sol.col_value, self.sol.col_dual, self.sol.row_dual

    def close(self):
        pass


CASES = [
    ("uniform", lambda: lpgen.planted_uniform(120, 300, 5, seed=21),
     {"pdhg_tolerance": 1e-7, "random_seed": 3}),
    ("maximise", lambda: lpgen.planted_general(30, 45, 3, seed=101, maximize=True, free=False),
     {"pdhg_tolerance": 1e-6, "iteration_limit": 50000}),
    ("no_restarts", lambda: lpgen.planted_uniform(60, 150, 5, seed=9),
     {"pdhg_tolerance": 1e-8, "pdhg_restart": False, "iteration_limit": 2000}),
    ("stop_at_request", lambda: lpgen.planted_uniform(60, 150, 5, seed=9),
     {"pdhg_tolerance": 1e-6, "pdhg_stop_at_request": True}),
    ("time_limit_zero", lambda: lpgen.planted_uniform(40, 90, 3, seed=2), {"time_limit": 0.0}),
    ("defaults", lambda: from_dense([[1, 1]], [2], [INF], [1, 1]), {}),
]


@pytest.mark.parametrize("name,make,options", CASES, ids=[c[0] for c in CASES])
def test_mirror_returns_the_oracles_answer(built, oracle, name, make, options):
    lp = make()
    eng = OracleEngine(oracle)
    got = capi.solve_pdhg_gpu(lp, options, engine=eng)
    call = eng.calls[-1]
    want = oracle.solve(lp, tolerance=call["tolerance"], iteration_limit=call["iteration_limit"],
                        time_limit=call["time_limit"], restart=call["restart"],
                        stop_at_request=call["stop_at_request"],
                        random_seed=call["random_seed"])
    assert got.status == want.status_name
    assert got.iterations == want.iterations
    assert got.objective == want.objective
    assert got.dual_bound == want.dual_bound or (np.isinf(got.dual_bound)
                                                 and np.isinf(want.dual_bound))
    assert np.array_equal(got.col_value, want.col_value)
    assert np.array_equal(got.col_dual, want.col_dual)
    assert np.array_equal(got.row_dual, want.row_dual)
    assert got.algorithm == "pdhg-gpu"
    expected = {"pdhg_tolerance": ("tolerance", 1e-4), "iteration_limit": ("iteration_limit", -1),
                "time_limit": ("time_limit", None), "pdhg_restart": ("restart", True),
                "pdhg_stop_at_request": ("stop_at_request", False),
                "random_seed": ("random_seed", 0)}
    for option, (arg, default) in expected.items():
        assert call[arg] == options.get(option, default), (option, call[arg])


def test_model_defect_is_a_status(built, oracle):
    lp = lpgen.planted_uniform(20, 40, 3, seed=1)
    lp.values = lp.values.copy()
    lp.values[5] = np.nan
    sol = capi.solve_pdhg_gpu(lp, {}, engine=OracleEngine(oracle))
    assert sol.status == "model_error" and sol.message
    assert sol.col_value.shape == (lp.cols,) and sol.row_dual.shape == (lp.rows,)


class OracleQpEngine:
    """QpEngine's interface over the oracle's QP restatement. Records each solve's settings."""

    def __init__(self, oracle):
        self.oracle = oracle
        self.calls = []

    def load(self, qp):
        diag = [qp.hessian_values[k] * qp.lp.sense for j in range(qp.cols)
                for k in range(qp.hessian_starts[j], qp.hessian_starts[j + 1])
                if qp.hessian_index[k] == j]
        if any(v < -1e-10 * max(1.0, max(abs(u) for u in diag)) for v in diag):
            raise capi.EngineError(3, "the quadratic objective is not convex: a negative "
                                      "diagonal")
        self.qp = qp

    def solve(self, tolerance, iteration_limit, time_limit, random_seed, interrupt=None,
              log=None):
        from types import SimpleNamespace

        self.calls.append(dict(tolerance=tolerance, iteration_limit=iteration_limit,
                               time_limit=time_limit, random_seed=random_seed))
        self.last = self.oracle.solve_qp(self.qp, tolerance=tolerance,
                                         iteration_limit=iteration_limit,
                                         time_limit=time_limit, random_seed=random_seed)
        return SimpleNamespace(status_name=self.last.status_name,
                               objective=self.last.objective, iterations=self.last.iterations,
                               message="")

    def solution(self):
        return self.last.col_value, self.last.col_dual, self.last.row_dual

    def close(self):
        pass


@pytest.mark.parametrize("options", [
    None,
    {"qp_tolerance": 1e-6, "iteration_limit": 777, "random_seed": 3},
    {"qp_tolerance": 1e-9, "time_limit": 0.0},
], ids=["defaults", "set", "time0"])
def test_qp_mirror_passes_the_options(built, oracle, options):
    """solve_convex_qp_gpu hands the registry's QP rows (and their defaults) to the engine and
    returns its point, with the bound only when optimal."""
    from sankhya_gb300.model import random_qp

    qp = random_qp(81, 30, 60, maximise=options is not None)
    eng = OracleQpEngine(oracle)
    s = capi.solve_convex_qp_gpu(qp, options, engine=eng)
    want = {"tolerance": 1e-8, "iteration_limit": -1, "time_limit": None, "random_seed": 0}
    for k, v in (options or {}).items():
        want[{"qp_tolerance": "tolerance"}.get(k, k)] = v
    assert eng.calls == [want]
    o = oracle.solve_qp(qp, **{k: v for k, v in want.items() if v is not None})
    assert (s.status, s.iterations) == (o.status_name, o.iterations)
    assert np.array_equal(s.col_value, o.col_value) and np.array_equal(s.row_dual, o.row_dual)
    assert s.algorithm == "qp-condat-vu-gpu"
    if s.status == "optimal":
        assert s.dual_bound == s.objective
    else:
        assert s.dual_bound == (np.inf if qp.lp.sense < 0 else -np.inf)


def test_qp_mirror_model_error(built, oracle):
    from sankhya_gb300.model import qp_from_dense

    qp = qp_from_dense([0.0, 0.0], [-INF, -INF], [INF, INF], [(0, 0, 1.0), (1, 1, -1.0)])
    s = capi.solve_convex_qp_gpu(qp, engine=OracleQpEngine(oracle))
    assert s.status == "model_error" and "not convex" in s.message

"""Committed outputs of the reference's own PDHG (tests/golden/reference_pdhg.json, made by
tests/golden/make_golden.py from oracle/_ref) pin both the oracle and the GPU engine on
machines where the reference sources are absent.

* The oracle must reproduce them bit-for-bit (status, iterations, restarts, objective,
  dual bound, the three returned vectors) on x86-64, where the fixtures were made; on other
  hosts libm's pow/exp/log may round differently, so there the trajectory may drift and the
  check falls back to the engine's bar.
* The GPU engine must give the same status and the objective within 1e-6 relative.
"""
import hashlib
import json
import os
import platform

import numpy as np
import pytest

from sankhya_gb300 import capi, lpgen

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_pdhg.json")) as f:
    GOLDEN = json.load(f)["cases"]


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def rebuild(case):
    lp = getattr(lpgen, case["generator"])(**case["args"])
    assert digest(lp.col_starts, lp.row_index, lp.values, lp.col_cost, lp.col_lower,
                  lp.col_upper, lp.row_lower, lp.row_upper) == case["instance_sha256"], \
        "the generator no longer rebuilds this instance bit-for-bit"
    return lp


def _id(case):
    a = case["args"]
    return f"{case['generator']}_{a.get('m', a.get('blocks'))}_s{a['seed']}_" + \
        "_".join(f"{k}{v}" for k, v in sorted(case["options"].items()))


@pytest.mark.parametrize("case", GOLDEN, ids=[_id(c) for c in GOLDEN])
def test_oracle_reproduces_reference(built, oracle, case):
    lp = rebuild(case)
    s = oracle.solve(lp, **case["options"])
    assert s.status_name == case["status"]
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("bit-level trajectory pinned on x86-64 only (libm rounding)")
    assert s.iterations == case["iterations"]
    if case["restarts"] >= 0:
        assert s.restarts == case["restarts"]
    assert float(s.objective).hex() == case["objective"]
    assert float(s.dual_bound).hex() == case["dual_bound"]
    assert digest(s.col_value) == case["col_value_sha256"]
    assert digest(s.col_dual) == case["col_dual_sha256"]
    assert digest(s.row_dual) == case["row_dual_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=[_id(c) for c in GOLDEN])
def test_engine_matches_reference_outputs(engine, case):
    lp = rebuild(case)
    o = case["options"]
    sol = capi.solve_pdhg_gpu(lp, {"pdhg_tolerance": o["tolerance"],
                                   "iteration_limit": o.get("iteration_limit", -1),
                                   "pdhg_restart": o.get("restart", True),
                                   "pdhg_stop_at_request": o.get("stop_at_request", False)},
                              engine=engine)
    if o.get("stop_at_request"):
        assert sol.status in ("optimal", "feasible")
    else:
        assert sol.status == case["status"], sol.message
    if case["status"] == "iteration_limit":
        assert sol.iterations == case["iterations"]
        return
    ref_obj = case["objective_float"]
    assert abs(sol.objective - ref_obj) <= 1e-6 * max(1.0, abs(ref_obj))

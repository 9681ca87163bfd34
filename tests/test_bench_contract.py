"""The bench's JSON line, on the CPU.

`bench.main()` runs with the device engines replaced by stand-ins that return fixed results
(the batched engine's stand-in solves the adjoint section's LPs exactly at their planted
basis), on a small block-angular LP and small batches. The CPU legs (the oracle baseline, the
reference arm) run for real. The test checks that every key the line promises is present and
well-formed, for the default arm and for `--impl reference`. It checks the line's assembly;
the numbers come from the GPU runs.
"""
import contextlib
import io
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "sih-26_gb300", "oracle", "tests"):
    sys.path.insert(0, os.path.join(ROOT, sub))

pytest.importorskip("scipy.sparse")


class _Result:
    def __init__(self, lp, precision="mixed"):
        self.status_name = "feasible"
        self.iterations = 400
        self.attempts = 402
        self.refinements = 3 if precision == "mixed" else 0
        self.restarts = 2
        self.objective = lp.fstar if lp.fstar is not None else 0.0
        self.residuals = {"primal": 1e-9, "dual": 2e-9, "gap": 3e-9}
        self.setup_seconds = 0.01
        self.loop_seconds = 0.08
        self.device_seconds = 0.09
        self.kernel_launches = 1000
        self.staged_fraction = (0.99, 0.0)


class StandInPdhgEngine:
    def __init__(self, device=0):
        self.lp = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def load(self, lp):
        self.lp = lp

    def solve(self, precision="fp64", **kw):
        return _Result(self.lp, precision)

    def time_kernels(self, reps):
        return 0.08, 0.1

    def solution(self):
        return np.zeros(self.lp.cols), np.zeros(self.lp.cols), np.zeros(self.lp.rows)

    def close(self):
        pass


class StandInQpEngine:
    """The QP engine's calls answered by the oracle's restatement (the answers the bench's
    same-answer check compares are then the oracle's own, so the check must pass)."""

    def __init__(self, device=0):
        import pyoracle

        self.oracle = pyoracle.Oracle()
        self.last = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def load(self, qp):
        self.qp = qp

    def solve(self, tolerance=1e-8, iteration_limit=-1, **kw):
        from types import SimpleNamespace

        self.last = self.oracle.solve_qp(self.qp, tolerance=tolerance,
                                         iteration_limit=iteration_limit)
        return SimpleNamespace(status_name=self.last.status_name,
                               iterations=self.last.iterations, device_seconds=0.2,
                               setup_seconds=0.01, loop_seconds=0.19, column_lanes=1,
                               row_lanes=2, kernel_launches=10, primal_residual=1e-3,
                               dual_residual=1e-4)

    def time_kernels(self, reps):
        return 0.05, 0.04

    def solution(self):
        return self.last.col_value, self.last.col_dual, self.last.row_dual

    def close(self):
        pass


def _batch_engine():
    from test_bench_adjoint_check import ExactBatchEngine, _Item

    class StandInBatchEngine(ExactBatchEngine):
        """Exact on LPs with a square planted basis (the adjoint section's), fixed items
        otherwise (the batched section's)."""

        def load(self, lps):
            self.lps = list(lps)
            for lp in self.lps:
                if getattr(lp, "x0", None) is not None:
                    basic = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
                    if int(basic.sum()) == lp.rows:
                        ExactBatchEngine.bases[id(lp.values)] = (basic, lp.x0 <= lp.col_lower)

        def solve(self, **kw):
            if all(id(lp.values) in ExactBatchEngine.bases for lp in self.lps):
                return super().solve(**kw)
            return [_Item(0.0) for _ in self.lps], 0.5

        def set_schedule(self, lanes=0, threads=0):
            self.schedule = (lanes, threads)

        def last_schedule(self):
            return 1, 256, 0.0

    return StandInBatchEngine


def _run(monkeypatch, argv):
    import bench
    from sankhya_gb300 import capi

    monkeypatch.setattr(capi, "PdhgEngine", StandInPdhgEngine)
    monkeypatch.setattr(capi, "QpEngine", StandInQpEngine)
    monkeypatch.setattr(bench, "QP_ITERATIONS", 300)
    monkeypatch.setattr(bench, "QP_CPU_SAMPLE", 7)
    monkeypatch.setattr(capi, "BatchEngine", _batch_engine())
    monkeypatch.setattr(bench, "WORKLOAD", dict(blocks=2, rows_per_block=300,
                                                cols_per_block=600, k=9, seed=2026))
    monkeypatch.setattr(bench, "BATCH_LPS", 6)
    monkeypatch.setattr(bench, "BATCH_NODES", 4)
    monkeypatch.setattr(bench, "BATCH_SEQUENTIAL_SAMPLE", (2, 1))
    monkeypatch.setattr(bench, "ZIPF_SHAPE", (300, 600, 3000))
    monkeypatch.setattr(bench, "REFERENCE_SAMPLE_ITERATIONS", 8)
    monkeypatch.setattr(bench, "CPU_TIME_LIMIT", 0.5)
    monkeypatch.setattr(bench, "reference_gpu_section",
                        lambda: {"ran_on_gpu": False, "s_per_iteration": 0.0})
    full_adjoint = bench.adjoint_section
    monkeypatch.setattr(bench, "adjoint_section",
                        lambda device: full_adjoint(device, lps_count=3, shape=(60, 120),
                                                    ref_lps=2, fd_lps=1, fd_coords=8))
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.main()
    lines = [l for l in buf.getvalue().splitlines() if l.startswith("{")]
    assert len(lines) == 1, buf.getvalue()
    return json.loads(lines[0])


def test_default_line(monkeypatch):
    line = _run(monkeypatch, ["--steps", "1", "--warmup", "3", "--cpu-iterations", "2"])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks", "fp64",
                "batched", "adjoint", "reference_gpu", "qp"):
        assert key in line, key
    qp = line["qp"]
    assert "error" not in qp, qp
    assert qp["iterations"] == 300 and qp["cpu"]["sample_iterations"] == 7
    assert qp["same_answer_at_sample"]["ok"] is True
    assert qp["column_pass_gbs"] == pytest.approx(qp["column_pass_bytes"] / 0.05 / 1e6)
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 3
    assert line["higher_is_better"] is False and line["unit"] == "s"
    assert "workload" in line["config"]
    roof = line["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    assert roof["traffic"] is None or roof["traffic"] > 0
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] > 0
    assert cpu["single_thread"].get("cores") == 1
    assert cpu["host"]["machine"] and cpu["host"]["logical_cpus"] >= cpu["cores"]
    e2e = line["e2e"]
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert line["gpu_launches"] > 0
    assert "error" not in line["batched"] and "error" not in line["adjoint"]
    assert set(line["batched"]) == {"independent", "bnb_nodes"}
    assert line["adjoint"]["fd_max_rel_err"] < 1e-5
    zipf = line["zipf"]
    assert "error" not in zipf, zipf
    for prec in ("mixed", "fp64"):
        assert zipf[prec]["relative_kkt"] >= 0 and zipf[prec]["seconds"] >= 0
    # The parity verdict and the FP64 summary close the line, where a reader that keeps only
    # its end still sees them.
    assert list(line)[-2:] == ["fp64", "parity"]
    parity = line["parity"]
    assert set(parity) >= {"mixed", "fp64", "objective_rel_diff_mixed_vs_fp64",
                           "speedup_of_mixed", "same_answer"}
    assert parity["same_answer"] is True
    limited = cpu["time_limited_run"]
    assert "error" not in limited and limited["time_limit_s"] == 0.5
    assert cpu["extrapolated"] is True
    assert e2e["pin_seconds"] >= 0 and e2e["value_with_pinning"] >= e2e["value"]


def test_reference_line(monkeypatch):
    line = _run(monkeypatch, ["--impl", "reference", "--steps", "1", "--warmup", "3",
                              "--cpu-iterations", "8"])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "s"
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["host"]["machine"]
    measured = line["cpu_baseline"]["measured"]
    assert measured["iterations"] == 8 and measured["s_per_iteration"] > 0
    assert line["cpu_baseline"]["extrapolated"] is True
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_pinned_inputs_are_exact_copies(monkeypatch):
    """bench.pinned_lp copies the LP into tensors allocated with pin_memory=True. Without a
    device here the allocation is made ordinary; the copy must still be exact and keep every
    dtype, and a failure anywhere must fall back to the LP itself."""
    torch = pytest.importorskip("torch")
    import bench
    from sankhya_gb300 import build, lpgen

    build.build_lpgen()
    lp = lpgen.planted_uniform(30, 70, 4, seed=2)
    real_empty = torch.empty
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(torch, "empty",
                        lambda *a, pin_memory=False, **k: real_empty(*a, **k))
    out, pinned = bench.pinned_lp(lp)
    assert pinned and out is not lp
    for name in ("col_starts", "row_index", "values", "col_cost", "col_lower", "col_upper",
                 "row_lower", "row_upper"):
        a, b = getattr(lp, name), getattr(out, name)
        assert b.dtype == a.dtype and np.array_equal(a, b), name
    assert (out.rows, out.cols, out.sense, out.objective_offset) == (lp.rows, lp.cols, lp.sense,
                                                                     lp.objective_offset)

    def fail(*a, **k):
        raise RuntimeError("no page-locked memory")

    monkeypatch.setattr(torch, "empty", fail)
    same, pinned = bench.pinned_lp(lp)
    assert same is lp and not pinned

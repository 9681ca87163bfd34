"""Benchmark: seconds to relative KKT 1e-8 for restarted PDHG on one GB300, mixed vs FP64.

Workload: the block-angular multi-period planted-optimum LP -- 64 periods of 15,625 rows x
31,250 columns, 9 N(0,1) entries per column inside its period plus one +-1 inventory link
into the next period: m = 1,000,000, n = 2,000,000, 19,968,750 nonzeros, 0 <= x <= 10,
equality rows (seeded synthetic data; the optimum f* = c.x0 is planted).

A STEP is one complete solve of that LP to relative KKT <= 1e-8 (max of the reference's
relative primal, dual and gap residuals on the unscaled problem) from the LP already
resident in HBM: device preconditioning, the PDHG loop, the exact FP64 evaluation. `value` is
the mixed-precision method's seconds per solve (CUDA events on the engine's stream, max over
ranks); the plain FP64 method is timed on the same LP beside it (`fp64`). The matrix (160-480
MB per value copy) is far larger than L2, so no L2 flush is needed between steps.

Also reported: each step kernel's achieved HBM GB/s against the measured copy bandwidth
(roofline), an end-to-end solve through the C ABI from host buffers (copies included), the
kernels launched, clocks sampled during the timed region, and the reference algorithm (the CPU
oracle on this host's cores) on a bounded sample, extrapolated to the FP64 iteration count.
Two further sections: `batched` -- LPs/s of the batched engine on 4,096 independent planted
LPs and on 1,024 branch-and-bound node relaxations of one 10,000 x 20,000 LP, against the
same LPs solved one at a time; `adjoint` -- 256 nondegenerate 5,000 x 10,000 LPs solved,
polished and differentiated, with the gradients checked against basis solves and finite
differences.

Multi-GPU: the path does not shard (one LP per device); N ranks run N independent replicas.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in ("sih-26_gb300", "oracle"):
    sys.path.insert(0, os.path.join(ROOT, sub))

METRIC = "sec to rel KKT 1e-8, mixed vs FP64 PDHG on 1 GB300; SpMV HBM GB/s; LPs/s"
WORKLOAD = dict(blocks=64, rows_per_block=15625, cols_per_block=31250, k=9, seed=2026)
TOLERANCE = 1e-8
# Accepted FP64 iterations to relative KKT 1e-8 on this workload (the FP64 method, whose
# step, restart and primal-weight rules are the reference's), measured by this bench's FP64
# solve on a GB300. The reference arm runs in a process of its own, without the GPU engine,
# so it projects its measured seconds per iteration with this count; the CPU baseline of the
# main arm uses the FP64 solve of the same run instead.
FP64_ITERATIONS_TO_1E8 = 115520
# CPU iterations each timed step of the reference arm measures: five evaluation points of the
# reference's 40-iteration cadence (src/pdhg/pdhg.cpp:341-384), so the sample includes the
# four unscaled products each evaluation adds.
REFERENCE_SAMPLE_ITERATIONS = 200
# The CPU baseline's run to 1e-8 under a time limit (seconds), as the plan for the large
# configs asks: its status and the relative KKT it reaches.
CPU_TIME_LIMIT = 30.0
# The load-balance stress LP (Zipf row lengths): each method runs to 1e-8 under this limit.
ZIPF_SHAPE = (500000, 1000000, 30000000)
ZIPF_TIME_LIMIT = 60.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes (read + write) of the step kernels at the full workload, from the
    committed ncu summary profiles/step_kernels_traffic.txt (lines "<kernel> <bytes>")."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "step_kernels_traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and not line.startswith("#"):
                    out[parts[0]] = float(parts[1])
    except OSError:
        pass
    return out


def algorithmic_bytes(m, n, nnz, v, w):
    """Per attempted step (the minimal fused form): column pass = (v+4) nnz + 4 (n+1)
    + w (m gathered + 7 n); row pass = (v+4) nnz + 4 (m+1) + w (2 n gathered + 6 m)."""
    col = (v + 4) * nnz + 4 * (n + 1) + w * (m + 7 * n)
    row = (v + 4) * nnz + 4 * (m + 1) + w * (2 * n + 6 * m)
    return col, row


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.seek(0)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def host_cpu():
    """The host's CPU model (lscpu's "Model name") and architecture, for the CPU baseline."""
    import platform

    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:  # noqa: BLE001 - a missing lscpu only loses the description
        pass
    return {"model": model, "machine": platform.machine(), "logical_cpus": os.cpu_count()}


# What the CPU baseline runs: the C restatement of the reference's PDHG, which the tests hold
# bit-identical to the reference's own sources compiled on x86-64.
CPU_BASELINE_PORT_OF = ("sankhya::pdhg::solve_pdhg (src/pdhg/pdhg.cpp) restated in C; "
                        "bit-identical to the reference's own build "
                        "(tests/test_oracle_vs_reference.py)")
CPU_BASELINE_REFERENCE = ("sankhya::pdhg::solve_pdhg (src/pdhg/pdhg.cpp), the reference's own "
                          "sources compiled on this host (oracle/_ref/libsankhya_ref.so)")


def pinned_lp(lp):
    """A copy of the LP whose arrays live in page-locked host memory, so that the end-to-end
    run copies its inputs to the device from pinned memory. Returns (lp, True), or the LP
    itself and False where torch has no CUDA device to pin with."""
    try:
        import numpy as np
        import torch
        from sankhya_gb300.model import LP

        if not torch.cuda.is_available():
            return lp, False
        keep = []

        def pin(a):
            a = np.ascontiguousarray(a)
            t = torch.empty(a.shape, dtype=getattr(torch, a.dtype.name), pin_memory=True)
            view = t.numpy()
            view[...] = a
            keep.append(t)
            return view

        out = LP(lp.rows, lp.cols, pin(lp.col_starts), pin(lp.row_index), pin(lp.values),
                 pin(lp.col_cost), pin(lp.col_lower), pin(lp.col_upper), pin(lp.row_lower),
                 pin(lp.row_upper), lp.sense, lp.objective_offset, name=lp.name)
        out.pinned_storage = keep  # the tensors that own the page-locked memory
        return out, True
    except Exception:  # noqa: BLE001 - pageable inputs still give an end-to-end number
        return lp, False


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def make_workload(blocks=None):
    from sankhya_gb300 import lpgen

    return lpgen.planted_blocks(blocks or WORKLOAD["blocks"], WORKLOAD["rows_per_block"],
                                WORKLOAD["cols_per_block"], WORKLOAD["k"], WORKLOAD["seed"])


def profile_qp(blocks):
    """The QP's small case for kernel captures: the same Hessian on a slice of `blocks`
    periods (32 periods: 500,000 x 1,000,000, about 1e7 nonzeros of A and 5e6 of Q: matrix
    copies of 120-180 MB), 200 iterations. Prints one line with the passes' CUDA-event times."""
    from sankhya_gb300 import build, capi

    build.build_lpgen()
    build.build_engine()
    qp = qp_workload(make_workload(blocks))
    col_bytes, row_bytes = qp_bytes(qp)
    with capi.QpEngine(0) as eng:
        eng.load(qp)
        r = eng.solve(tolerance=1e-30, iteration_limit=200)
        col_ms, row_ms = eng.time_kernels(20)
    print(json.dumps({"profile_qp": blocks, "status": r.status_name, "iterations": r.iterations,
                      "lanes": [r.column_lanes, r.row_lanes],
                      "column_pass_ms": col_ms, "row_pass_ms": row_ms,
                      "column_pass_gbs": col_bytes / col_ms / 1e6,
                      "row_pass_gbs": row_bytes / row_ms / 1e6}))


def profile_case(blocks, precision, iterations, zipf=False):
    """The small case the kernel captures run on: the same generator with fewer periods
    (16 periods: 250,000 x 500,000, about 5M nonzeros, matrix copies of 40-120 MB), solved for
    a fixed number of accepted iterations. With `zipf`, the load-balance stress LP instead:
    500,000 x 1,000,000, Zipf(1.5) row lengths, about 3e7 nonzeros, values of log-uniform
    magnitude over [1e-3, 1e3]. Prints one line (with the step kernels' CUDA-event times
    after the solve) and returns."""
    from sankhya_gb300 import build, capi, lpgen

    build.build_lpgen()
    build.build_engine()
    lp = (lpgen.planted_zipf(500000, 1000000, 30000000, seed=3) if zipf
          else make_workload(blocks))
    eng = capi.PdhgEngine(0)
    eng.load(lp)
    r = eng.solve(tolerance=TOLERANCE, stop_rule="relative", precision=precision,
                  iteration_limit=iterations, steps_per_poll=8)
    ms_primal, ms_dual = eng.time_kernels(20)
    v = 8 if precision == "fp64" else 4
    b_col, b_row = algorithmic_bytes(lp.rows, lp.cols, lp.nnz, v, v)
    print(json.dumps({"profile_case": f"{lp.rows} x {lp.cols}, {lp.nnz} nnz",
                      "precision": precision, "status": r.status_name,
                      "iterations": r.iterations, "staged_share": list(r.staged_fraction),
                      "us_per_attempt": 1e6 * r.loop_seconds / max(1, r.attempts),
                      "column_pass_us": 1e3 * ms_primal, "row_pass_us": 1e3 * ms_dual,
                      "column_pass_gbs": b_col / (ms_primal * 1e-3) / 1e9,
                      "row_pass_gbs": b_row / (ms_dual * 1e-3) / 1e9,
                      "relative_kkt": max(r.residuals["primal"], r.residuals["dual"],
                                          r.residuals["gap"])}))
    eng.close()


# Batched workloads: 4,096 independent planted LPs (m log-uniform in [50, 2,000], n = 2m,
# 5 nonzeros per column) and 1,024 branch-and-bound node relaxations of one planted
# 10,000 x 20,000 LP (1-20 bounds tightened to [0, floor x0_j] or [ceil x0_j, 10]).
BATCH_LPS = 4096
BATCH_NODES = 1024
BATCH_TOLERANCE = 1e-6
BATCH_SEQUENTIAL_SAMPLE = (64, 16)  # LPs of each part solved one at a time for the baseline


def make_batch_lps(seed=2027):
    from sankhya_gb300 import lpgen
    import numpy as np

    rng = np.random.default_rng(seed)
    ms = np.exp(rng.uniform(np.log(50), np.log(2000), size=BATCH_LPS)).astype(int)
    return [lpgen.planted_uniform(int(m), 2 * int(m), 5, seed=seed * 10000 + k)
            for k, m in enumerate(ms)]


def make_batch_nodes(seed=2028):
    from sankhya_gb300 import lpgen
    from sankhya_gb300.model import LP
    import numpy as np

    base = lpgen.planted_uniform(10000, 20000, 5, seed=seed)
    rng = np.random.default_rng(seed)
    nodes = []
    for _ in range(BATCH_NODES):
        lo, up = base.col_lower.copy(), base.col_upper.copy()
        for j in rng.choice(base.cols, size=int(rng.integers(1, 21)), replace=False):
            if rng.random() < 0.5:
                up[j] = np.floor(base.x0[j])
            else:
                lo[j] = np.ceil(base.x0[j])
        nodes.append(LP(base.rows, base.cols, base.col_starts, base.row_index, base.values,
                        base.col_cost, lo, up, base.row_lower, base.row_upper))
    return nodes


def batched_section(device):
    """LPs/s of the batched engine (mixed precision: FP32 iterations on FP64 refinement
    rounds, the schedule autotuned per batch) against the same LPs solved one at a time by the
    single-LP engine's plain FP64 method (a sample of each part, extrapolated); relative KKT
    <= 1e-6. Every independent LP's objective is held to its planted optimum, and every node
    relaxation reported infeasible has its Farkas certificate checked on the host."""
    from sankhya_gb300 import capi, certify

    out = {}
    for name, make, sample in (("independent", make_batch_lps, BATCH_SEQUENTIAL_SAMPLE[0]),
                               ("bnb_nodes", make_batch_nodes, BATCH_SEQUENTIAL_SAMPLE[1])):
        lps = make()
        with capi.BatchEngine(device) as eng:
            t0 = time.perf_counter()
            eng.load(lps)
            t_load = time.perf_counter() - t0
            items, dev_s = eng.solve(tolerance=BATCH_TOLERANCE, stop_rule="relative",
                                     iteration_limit=200000, precision="mixed")
            lanes, threads, tune_s = eng.last_schedule()
            rays = {k: eng.ray(k) for k, it in enumerate(items) if it.status_name == "infeasible"}
        statuses = {}
        for it in items:
            statuses[it.status_name] = statuses.get(it.status_name, 0) + 1
        step = max(1, len(lps) // sample)
        picked = lps[::step][:sample]
        seq_s = 0.0
        with capi.PdhgEngine(device) as one:
            for lp in picked:
                one.load(lp)
                r = one.solve(tolerance=BATCH_TOLERANCE, stop_rule="relative",
                              iteration_limit=200000)
                seq_s += r.device_seconds
        seq_rate = len(picked) / seq_s
        entry = {"lps": len(lps), "precision": "mixed", "device_s": dev_s, "load_s": t_load,
                 "schedule": {"lanes": lanes, "threads": threads, "autotune_s": tune_s},
                 "lps_per_s": len(lps) / dev_s, "statuses": statuses,
                 "iterations_mean": sum(it.iterations for it in items) / len(items),
                 "sequential_lps_per_s": seq_rate,
                 "sequential_sample": len(picked),
                 "speedup_vs_sequential": (len(lps) / dev_s) / seq_rate}
        if name == "independent":
            conv = [(it, lp) for it, lp in zip(items, lps) if it.converged]
            entry["objective_max_rel_err_vs_planted"] = max(
                (abs(it.objective - lp.fstar) / max(1.0, abs(lp.fstar)) for it, lp in conv),
                default=None)
        else:
            # Every node reported infeasible carries a Farkas ray, checked here in FP64 on the
            # host (exactly rounded sums); every other node must have converged.
            shares = [certify.farkas_share(lps[k], rays[k]) for k in rays]
            entry["infeasible_check"] = {
                "reported": len(rays), "certified": sum(1 for sh in shares if sh > 0.0),
                "min_share": min(shares, default=None),
                "not_converged_other": sum(1 for it in items
                                           if it.status_name != "infeasible" and not it.converged)}
        out[name] = entry
    return out


# Differentiation: 256 planted LPs of 5,000 x 10,000 with 5 nonzeros per column and a unique,
# nondegenerate optimum (the differentiable form of the planted generator), solved in one
# batch (mixed precision) and polished at their active sets, which puts x*, y* on the vertex
# in FP64; L = w'x* + v'y* + f* with w, v ~ N(0,1).
ADJOINT_LPS = 256
ADJOINT_SHAPE = (5000, 10000)
# The active sets of these LPs are settled long before PDHG's tail: the batch stops at this
# relative KKT and the polish puts x*, y* on the vertex (every LP is checked afterwards).
ADJOINT_FORWARD_TOLERANCE = 1e-4


def _basis_solver(device):
    """(solve_pair, description): solve_pair(S, a, b) returns (S'^-1 a, S^-1 b) for a square
    sparse S. A dense LU in FP64 on the device (cuSOLVER through torch) where CUDA is there,
    else SuperLU on the host: the reference basis solves of 256 LPs of 5,000 rows take
    seconds on the device and a quarter of an hour in SuperLU (its fill-in on these random
    bases reaches 8e6 entries)."""
    import numpy as np

    try:
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA")
        dev = torch.device("cuda", device)

        def solve_pair(S, a, b):
            D = torch.tensor(S.toarray(), dtype=torch.float64, device=dev)
            lu, piv = torch.linalg.lu_factor(D)
            rhs = torch.tensor(np.stack([a, b], axis=1), dtype=torch.float64, device=dev)
            p = torch.linalg.lu_solve(lu, piv, rhs[:, :1], adjoint=True)
            q = torch.linalg.lu_solve(lu, piv, rhs[:, 1:])
            return p[:, 0].cpu().numpy(), q[:, 0].cpu().numpy()

        return solve_pair, "dense LU in FP64 on the device (torch.linalg.lu_factor)"
    except Exception:  # noqa: BLE001
        import scipy.sparse.linalg as spl

        def solve_pair(S, a, b):
            lu = spl.splu(S.tocsc())
            return lu.solve(a, trans="T"), lu.solve(b)

        return solve_pair, "SuperLU on the host (scipy.sparse.linalg.splu)"


def adjoint_section(device, lps_count=ADJOINT_LPS, shape=ADJOINT_SHAPE, ref_lps=256, fd_lps=16,
                    fd_coords=64):
    """Forward + polish + adjoint times for the whole batch, and the gradients' agreement with
    (a) the basis solves of the planted optimum (sparse LU on the host, `ref_lps` LPs, every
    coordinate) and (b) central finite differences of L (step 1e-6) through re-solves of the
    perturbed LPs on the device (solve + polish, which land on the exact perturbed vertex), on
    `fd_coords` coordinates of `fd_lps` LPs spread over costs, right-hand sides and bounds."""
    import numpy as np
    from sankhya_gb300 import capi, lpgen
    from sankhya_gb300.model import LP

    m, n = shape
    lps = [lpgen.planted_nondegenerate(m, n, 5, seed=5000 + k) for k in range(lps_count)]
    rng = np.random.default_rng(4)
    gx = [rng.standard_normal(n) for _ in lps]
    gy = [rng.standard_normal(m) for _ in lps]
    solve_kw = dict(tolerance=ADJOINT_FORWARD_TOLERANCE, stop_rule="relative",
                    iteration_limit=2000000, precision="mixed")
    with capi.BatchEngine(device) as eng:
        eng.load(lps)
        items, fwd_s = eng.solve(**solve_kw)
        fwd_iterations = sum(it.iterations for it in items) / len(items)
        t0 = time.perf_counter()
        items, polish_info = eng.polish()
        polish_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        res = eng.adjoint(gx, gy, np.ones(len(lps)))
        adj_s = time.perf_counter() - t0
        vertex_err = 0.0
        base_points = {}
        for k in range(len(lps)):
            point = eng.solution(k)
            if k < fd_lps:
                base_points[k] = point
            if k < ref_lps:
                x, _, y = point
                vertex_err = max(vertex_err, float(np.abs(x - lps[k].x0).max()),
                                 float(np.abs(y - lps[k].lam).max()))
    out = {"lps": len(lps), "shape": [m, n], "forward_tolerance": ADJOINT_FORWARD_TOLERANCE,
           "forward_device_s": fwd_s, "polish_s": polish_s,
           "forward_iterations_mean": fwd_iterations,
           "adjoint_s": adj_s, "statuses": {}, "adjoint_status": {}, "cg_iterations_max": 0,
           "polished": sum(1 for p in polish_info if p["status"] == 0),
           "vertex_max_abs_err": vertex_err}
    for it, r in zip(items, res):
        out["statuses"][it.status_name] = out["statuses"].get(it.status_name, 0) + 1
        out["adjoint_status"][str(r["status"])] = out["adjoint_status"].get(str(r["status"]), 0) + 1
        out["cg_iterations_max"] = max(out["cg_iterations_max"], max(r["iterations"]))
    try:
        import scipy.sparse as sp
    except ImportError:
        out["basis_reference"] = "scipy unavailable"
    else:
        solve_pair, how = _basis_solver(device)
        out["basis_reference_solver"] = how
        worst = 0.0
        for lp, g_x, g_y, r in list(zip(lps, gx, gy, res))[:ref_lps]:
            A = sp.csc_matrix((lp.values, lp.row_index, lp.col_starts), shape=(m, n))
            B = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
            p, q = solve_pair(A[:, B], g_x[B], g_y)
            d = lp.col_cost - A.T @ lp.lam
            dc = lp.x0.copy()
            dc[B] += q
            db = p + lp.lam
            dbound = g_x - A.T @ p + d
            dl = np.where(~B & (lp.x0 <= lp.col_lower), dbound, 0.0)
            du = np.where(~B & (lp.x0 >= lp.col_upper), dbound, 0.0)
            for got, want in ((r["dc"], dc), (r["drl"] + r["dru"], db), (r["dl"], dl),
                              (r["du"], du)):
                worst = max(worst,
                            float(np.max(np.abs(got - want) / np.maximum(1.0, np.abs(want)))))
        out["max_rel_err_vs_basis_solves"] = worst
        out["basis_reference_lps"] = min(ref_lps, len(lps))
    # Finite differences: perturbed copies (sharing each LP's matrix) re-solved in one batch,
    # 64 coordinates per LP: 16 costs, 16 right-hand sides, 16 lower bounds of columns at
    # their lower bound and 16 upper bounds of columns at their upper bound (the bounds that
    # move the optimum). The loss difference is summed from the solutions' differences, so
    # the two nearly equal losses are never subtracted.
    h = 1e-6
    per_family = fd_coords // 4
    pert, meta = [], []
    for k in range(min(fd_lps, len(lps))):
        lp = lps[k]
        at_l = np.flatnonzero(lp.x0 <= lp.col_lower)
        at_u = np.flatnonzero(lp.x0 >= lp.col_upper)
        picks = ([("c", int(j)) for j in rng.choice(n, per_family, replace=False)] +
                 [("b", int(i)) for i in rng.choice(m, per_family, replace=False)] +
                 [("l", int(j)) for j in rng.choice(at_l, min(per_family, at_l.size), replace=False)] +
                 [("u", int(j)) for j in rng.choice(at_u, min(per_family, at_u.size), replace=False)])
        for fam, j in picks:
            for sign in (1.0, -1.0):
                c, lo, up = lp.col_cost.copy(), lp.col_lower.copy(), lp.col_upper.copy()
                rl, ru = lp.row_lower.copy(), lp.row_upper.copy()
                if fam == "c":
                    c[j] += sign * h
                elif fam == "b":
                    rl[j] += sign * h
                    ru[j] += sign * h
                elif fam == "l":
                    lo[j] += sign * h
                else:
                    up[j] += sign * h
                pert.append(LP(m, n, lp.col_starts, lp.row_index, lp.values, c, lo, up, rl, ru))
                meta.append((k, fam, j, sign))
    # Each perturbed LP is solved by PDHG and then polished from its base LP's vertex (a warm
    # start, sankhya_gb300_batch_set_point): the polish re-solves the base's active sets for
    # the perturbed data, so the +h and -h vertices carry the same rounding (the basis
    # matrices' condition numbers reach 1e5 here, so two independently polished vertices
    # differ by up to ~1e-9 of rounding, which a step of 1e-6 would turn into ~1e-3).
    with capi.BatchEngine(device) as eng:
        eng.load(pert)
        eng.solve(**solve_kw)
        for q, (k, _, _, _) in enumerate(meta):
            eng.set_point(q, *base_points[k])
        fitems, finfo = eng.polish()
        sols = [eng.solution(q) for q in range(len(meta))]
    fd_worst, fam_worst, fd_count = 0.0, {}, 0
    for q in range(0, len(meta), 2):
        k, fam, j, _ = meta[q]
        lp = lps[k]
        (xp, _, yp), (xm, _, ym) = sols[q], sols[q + 1]
        dx, dy = xp - xm, yp - ym
        dl = (gx[k] + lp.col_cost) @ dx + gy[k] @ dy
        if fam == "c":
            dl += h * (xp[j] + xm[j])
        fd = dl / (2 * h)
        r = res[k]
        if fam == "c":
            got = r["dc"][j]
        elif fam == "b":
            got = r["drl"][j] + r["dru"][j]
        else:
            got = r["dl" if fam == "l" else "du"][j]
        err = abs(got - fd) / max(1.0, abs(fd))
        fd_worst = max(fd_worst, err)
        fam_worst[fam] = max(fam_worst.get(fam, 0.0), err)
        fd_count += 1
    out["fd_max_rel_err"] = fd_worst
    out["fd_max_rel_err_by_family"] = fam_worst
    out["fd_polished"] = sum(1 for p in finfo if p["status"] == 0)
    out["fd_sample"] = (f"{min(fd_lps, len(lps))} LPs x {fd_count // max(1, min(fd_lps, len(lps)))} "
                        f"coordinates (costs, right-hand sides, active lower and upper bounds), "
                        f"central differences with step {h}; the {len(meta)} perturbed LPs "
                        f"re-solved in one batch and polished from their base LP's vertex")
    return out


def zipf_section(device, peak):
    """The load-balance stress LP (500,000 x 1,000,000, Zipf(1.5) row lengths, about 3e7
    nonzeros, badly scaled values): each method to relative KKT 1e-8 under ZIPF_TIME_LIMIT
    seconds, with the status and KKT it reaches, its objective against the planted optimum,
    and its step kernels' achieved bandwidth."""
    from sankhya_gb300 import capi, lpgen

    m, n, z = ZIPF_SHAPE
    lp = lpgen.planted_zipf(m, n, z, seed=3)
    out = {"shape": [lp.rows, lp.cols], "nnz": lp.nnz, "time_limit_s": ZIPF_TIME_LIMIT}
    with capi.PdhgEngine(device) as eng:
        eng.load(lp)
        for prec in ("mixed", "fp64"):
            r = eng.solve(tolerance=TOLERANCE, stop_rule="relative", precision=prec,
                          time_limit=ZIPF_TIME_LIMIT)
            k = kernel_roofline(eng, lp, prec, peak, r.staged_fraction)
            out[prec] = {"status": r.status_name, "seconds": r.device_seconds,
                         "iterations": r.iterations, "relative_kkt": relative_kkt(r.residuals),
                         "objective_rel_err": abs(r.objective - lp.fstar) / max(1.0, abs(lp.fstar)),
                         "us_per_attempt": 1e6 * r.loop_seconds / max(1, r.attempts),
                         "k_primal_gbs": k["k_primal_gbs"], "k_dual_gbs": k["k_dual_gbs"],
                         "k_primal_frac": k["k_primal_frac"], "k_dual_frac": k["k_dual_frac"]}
    return out


# The convex QP on the same kernels' terms (src/qp/qp_condat_vu.cpp): the 1M x 2M LP's rows,
# columns and cost with a banded positive definite Hessian (two sub-diagonals, a dominant
# diagonal; 6M stored entries, 10M in the full symmetric Q). Condat-Vu has a fixed step and
# no restarts, so the GPU leg is a fixed QP_ITERATIONS at a tolerance no run meets, and the
# reference's CPU engine is timed on QP_CPU_SAMPLE iterations of the same QP.
QP_HESSIAN = dict(band=2, seed=7)
QP_ITERATIONS = 2000
QP_CPU_SAMPLE = 20


def qp_workload(lp):
    from sankhya_gb300.model import QP, banded_hessian

    hs, hi, hv = banded_hessian(lp.cols, QP_HESSIAN["band"], seed=QP_HESSIAN["seed"])
    return QP(lp, hs, hi, hv, "qp_" + lp.name)


def qp_bytes(qp):
    """Algorithmic bytes of one column and one row pass: matrix values and indices (A's
    column and Q's full rows; A's rows), both passes' pointer arrays, each gathered vector
    once, each streamed vector once (column pass: c, l, u, x read, x' and xbar written; row
    pass: rl, ru, y read, y written)."""
    m, n = qp.rows, qp.cols
    za = qp.lp.nnz
    zq = 2 * qp.hessian_nnz - n
    col = 12 * (za + zq) + 8 * (n + 1) + 8 * n + 8 * m + 32 * n + 16 * n
    row = 12 * za + 4 * (m + 1) + 8 * n + 24 * m + 8 * m
    return col, row


def qp_section(device, peak, lp, cpu=True):
    """The convex QP: GPU iterations per second over QP_ITERATIONS, its column and row
    passes' achieved bandwidth (CUDA events, 20 iterations), the reference's CPU engine per
    iteration on QP_CPU_SAMPLE iterations, and the same-answer check at that count."""
    import numpy as np
    from sankhya_gb300 import capi

    qp = qp_workload(lp)
    col_bytes, row_bytes = qp_bytes(qp)
    out = {"workload": f"QP {qp.rows:,} x {qp.cols:,}: the LP's rows and bounds, {lp.nnz:,} "
                       f"nonzeros of A, a banded Hessian of {qp.hessian_nnz:,} stored "
                       f"({2 * qp.hessian_nnz - qp.cols:,} full) entries",
           "iterations": QP_ITERATIONS}
    with capi.QpEngine(device) as eng:
        t0 = time.perf_counter()
        eng.load(qp)
        out["load_s"] = time.perf_counter() - t0
        eng.solve(tolerance=1e-30, iteration_limit=100)  # warm-up (graph capture)
        r = eng.solve(tolerance=1e-30, iteration_limit=QP_ITERATIONS)
        col_ms, row_ms = eng.time_kernels(20)
        out.update({"status": r.status_name, "device_s": r.device_seconds,
                    "setup_s": r.setup_seconds, "loop_s": r.loop_seconds,
                    "us_per_iteration": 1e6 * r.loop_seconds / max(1, r.iterations),
                    "iterations_per_s": r.iterations / r.loop_seconds if r.loop_seconds else None,
                    "lanes": [r.column_lanes, r.row_lanes], "kernel_launches": r.kernel_launches,
                    "primal_residual": r.primal_residual, "dual_residual": r.dual_residual,
                    "column_pass_ms": col_ms, "row_pass_ms": row_ms,
                    "column_pass_bytes": col_bytes, "row_pass_bytes": row_bytes,
                    "column_pass_gbs": col_bytes / col_ms / 1e6,
                    "row_pass_gbs": row_bytes / row_ms / 1e6,
                    "column_pass_frac": col_bytes / col_ms / 1e6 / peak,
                    "row_pass_frac": row_bytes / row_ms / 1e6 / peak})
        if cpu:
            threads = os.cpu_count() or 1
            o = _oracle(threads)
            t0 = time.perf_counter()
            o.solve_qp(qp, tolerance=1e-30, iteration_limit=0)
            setup = time.perf_counter() - t0
            t0 = time.perf_counter()
            c = o.solve_qp(qp, tolerance=1e-30, iteration_limit=QP_CPU_SAMPLE)
            per_it = max(time.perf_counter() - t0 - setup, 0.0) / QP_CPU_SAMPLE
            g = eng.solve(tolerance=1e-30, iteration_limit=QP_CPU_SAMPLE)
            x, d, y = eng.solution()

            def rel(a, b):
                return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))

            out["cpu"] = {"kind": cpu_kind()[0],
                          "engine": "sankhya::qp::solve_convex_qp (src/qp/qp_condat_vu.cpp)"
                                    + (", the reference's own build" if cpu_kind()[0] ==
                                       "reference" else ", the oracle's C restatement"),
                          "cores": threads, "setup_s": setup, "s_per_iteration": per_it,
                          "sample_iterations": QP_CPU_SAMPLE,
                          "speedup_per_iteration": per_it / (1e-6 * out["us_per_iteration"])}
            out["same_answer_at_sample"] = {
                "iterations": [g.iterations, c.iterations],
                "x_rel_diff": rel(x, c.col_value), "col_dual_rel_diff": rel(d, c.col_dual),
                "row_dual_rel_diff": rel(y, c.row_dual),
                "ok": bool(g.iterations == c.iterations and rel(x, c.col_value) <= 1e-9
                           and rel(d, c.col_dual) <= 1e-9 and rel(y, c.row_dual) <= 1e-9)}
    return out


# The north star's "same answer": both methods' objectives within 1e-6 relative of each
# other and of the planted optimum, and each at relative KKT <= 1e-8 by the exact FP64
# evaluation of the reference's residuals (src/pdhg/pdhg_evaluate.hpp:48).
PARITY_OBJECTIVE = 1e-6


def parity_object(lp, mixed, fp64, mixed_s, fp64_s):
    def one(r):
        return {"status": r.status_name, "iterations": r.iterations,
                "relative_kkt": relative_kkt(r.residuals),
                "objective_rel_err": abs(r.objective - lp.fstar) / max(1.0, abs(lp.fstar))}

    out = {"mixed": one(mixed)}
    ok = out["mixed"]["relative_kkt"] <= TOLERANCE and \
        out["mixed"]["objective_rel_err"] <= PARITY_OBJECTIVE
    if fp64 is not None:
        out["fp64"] = one(fp64)
        diff = abs(mixed.objective - fp64.objective) / max(1.0, abs(fp64.objective))
        out["objective_rel_diff_mixed_vs_fp64"] = diff
        out["speedup_of_mixed"] = fp64_s / mixed_s
        ok = ok and out["fp64"]["relative_kkt"] <= TOLERANCE and \
            out["fp64"]["objective_rel_err"] <= PARITY_OBJECTIVE and diff <= PARITY_OBJECTIVE
    out["same_answer"] = bool(ok)
    return out


def workload_config(lp, precision):
    return {"workload": f"block-angular planted LP {lp.rows:,} x {lp.cols:,}, {lp.nnz:,} nnz, "
                        f"{WORKLOAD['blocks']} periods, seed {WORKLOAD['seed']}",
            "tolerance": TOLERANCE, "precision": precision,
            "stopping": "relative KKT <= 1e-8 (pdhg_stop_rule=relative)",
            "step": "one complete solve from the HBM-resident LP",
            "l2": "inputs larger than L2 (matrix values 160-480 MB per copy); no flush"}


def _oracle(threads):
    """The CPU implementation the baselines time: the reference's own PDHG compiled from its
    sources (oracle/_ref, built by __graft_entry__.build from the reference tree or its staged
    copy) where it is built, else the oracle's C restatement of it."""
    import ctypes
    import pyoracle

    pyoracle.build()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    try:  # the oracle's OpenMP runtime is shared with this process once loaded
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(threads))
    except (OSError, AttributeError):
        pass
    return pyoracle.Oracle(reference=pyoracle.reference_available())


def cpu_kind():
    """("reference", what it is) when the reference's own build is there, else ("port", ...)."""
    import pyoracle

    if pyoracle.reference_available():
        return "reference", CPU_BASELINE_REFERENCE
    return "port", CPU_BASELINE_PORT_OF


def relative_kkt(residuals):
    return max(residuals["primal"], residuals["dual"], residuals["gap"])


def cpu_reference(lp, iterations_sample, threads):
    """The reference algorithm on this host: the oracle (C restatement, OpenMP A^T y like the
    reference) -- setup alone, then setup + `iterations_sample` iterations. Returns (setup
    seconds, seconds per iteration, seconds of CPU work, the sample's result)."""
    o = _oracle(threads)
    t0 = time.perf_counter()
    o.solve(lp, tolerance=TOLERANCE, iteration_limit=0)
    setup = time.perf_counter() - t0
    if iterations_sample <= 0:
        return setup, 0.0, setup, None
    t0 = time.perf_counter()
    r = o.solve(lp, tolerance=TOLERANCE, iteration_limit=iterations_sample)
    sampled = time.perf_counter() - t0
    per_it = max(sampled - setup, 0.0) / max(1, r.iterations)
    if per_it <= 0.0:
        # An LP so small that the sample's iterations are lost in the setup's timing noise:
        # the whole sample per iteration, an upper bound.
        per_it = sampled / max(1, r.iterations)
    return setup, per_it, sampled + setup, r


def cpu_time_limited(lp, threads, time_limit):
    """The oracle run to relative KKT 1e-8 under a time limit: what it reaches."""
    o = _oracle(threads)
    t0 = time.perf_counter()
    r = o.solve(lp, tolerance=TOLERANCE, time_limit=time_limit)
    return {"time_limit_s": time_limit, "wall_s": time.perf_counter() - t0,
            "status": r.status_name, "iterations": r.iterations,
            "relative_kkt": relative_kkt(r.residuals), "objective": r.objective}


# The reference's own CUDA PDHG (src/gpu/pdhg_gpu.cu, built from its sources by
# `make -C oracle ref-gpu`): the existing-GPU bar. It runs in a child process, so that its
# device memory and any failure of it stay out of this process.
REFERENCE_GPU_TIME_LIMIT = 150.0
REFERENCE_GPU_SAMPLE_ITERATIONS = 2000

_REFERENCE_GPU_CHILD = r"""
import json, sys, time
sys.path[:0] = [sys.argv[1], sys.argv[2]]
import bench, pyoracle
lp = bench.make_workload()
out = {}
for key, kw in (("setup", dict(iteration_limit=0)),
                ("sample", dict(iteration_limit=int(sys.argv[3]))),
                ("to_1e8", dict(time_limit=float(sys.argv[4])))):
    t0 = time.perf_counter()
    r = pyoracle.reference_gpu_solve(lp, bench.TOLERANCE, **kw)
    r["wall_s"] = time.perf_counter() - t0
    r["objective_rel_err"] = abs(r["objective"] - lp.fstar) / max(1.0, abs(lp.fstar))
    out[key] = r
print("REFGPU " + json.dumps(out))
"""


def reference_gpu_section():
    """The reference's CUDA PDHG on the 1M x 2M LP: its setup alone (iteration limit 0), a
    fixed sample of iterations, and a run to tolerance 1e-8 under its own stopping rule and
    REFERENCE_GPU_TIME_LIMIT; seconds per iteration from the first two."""
    import pyoracle

    t0 = time.perf_counter()
    pyoracle.build_reference_gpu()
    build_s = time.perf_counter() - t0
    proc = subprocess.run([sys.executable, "-c", _REFERENCE_GPU_CHILD, os.path.dirname(
        os.path.abspath(__file__)), os.path.dirname(os.path.abspath(pyoracle.__file__)),
        str(REFERENCE_GPU_SAMPLE_ITERATIONS), str(REFERENCE_GPU_TIME_LIMIT)],
        capture_output=True, text=True, timeout=REFERENCE_GPU_TIME_LIMIT + 600)
    lines = [l for l in proc.stdout.splitlines() if l.startswith("REFGPU ")]
    if proc.returncode != 0 or not lines:
        return {"error": f"exit {proc.returncode}: {(proc.stderr or proc.stdout)[-400:]}"}
    runs = json.loads(lines[-1][len("REFGPU "):])
    setup, sample, full = runs["setup"], runs["sample"], runs["to_1e8"]
    per_it = max(sample["solve_seconds"] - setup["solve_seconds"], 0.0) / max(
        1, sample["iterations"])
    statuses = {1: "optimal", 5: "feasible", 6: "iteration_limit", 7: "time_limit",
                9: "numerical_error"}
    # An unconverged run states its relative residuals in the message ("stopped at relative
    # primal P, dual D, gap G ...", src/gpu/pdhg_gpu.cu:796-799); a converged one met the
    # request (relative KKT <= the tolerance) by definition.
    import re

    rel = re.search(r"relative primal ([0-9.e+-]+), dual ([0-9.e+-]+), gap ([0-9.e+-]+)",
                    full["message"])
    full_kkt = max(float(v) for v in rel.groups()) if rel else None
    return {"engine": "src/gpu/pdhg_gpu.cu (cuSPARSE SpMV + its elementwise kernels), FP64",
            "ran_on_gpu": all(r["algorithm"] == "pdhg-cuda" for r in runs.values()),
            "build_s": build_s, "setup_s": setup["solve_seconds"],
            "s_per_iteration": per_it, "sample_iterations": sample["iterations"],
            "to_1e8": {"status": statuses.get(full["status"], str(full["status"])),
                       "seconds": full["solve_seconds"], "iterations": full["iterations"],
                       "time_limit_s": REFERENCE_GPU_TIME_LIMIT,
                       "met_request": full["status"] in (1, 5), "relative_kkt": full_kkt,
                       "primal_infeasibility": full["primal_infeasibility"],
                       "dual_infeasibility": full["dual_infeasibility"],
                       "objective_rel_err": full["objective_rel_err"],
                       "message": full["message"][:200]}}


def kernel_roofline(eng, lp, precision, peak, staged=None):
    """Mean CUDA-event durations of the two step passes (on the engine's stream, 20 steps on
    the state the last solve left) and their achieved GB/s on the algorithmic bytes."""
    ms_primal, ms_dual = eng.time_kernels(20)
    v = w = 8 if precision == "fp64" else 4
    b_col, b_row = algorithmic_bytes(lp.rows, lp.cols, lp.nnz, v, w)
    return {"k_primal_ms": ms_primal, "k_dual_ms": ms_dual,
            "staged_share": list(staged) if staged is not None else None,
            "k_primal_gbs": b_col / (ms_primal * 1e-3) / 1e9,
            "k_dual_gbs": b_row / (ms_dual * 1e-3) / 1e9,
            "k_primal_bytes": b_col, "k_dual_bytes": b_row,
            "k_primal_frac": b_col / (ms_primal * 1e-3) / 1e9 / peak,
            "k_dual_frac": b_row / (ms_dual * 1e-3) / 1e9 / peak}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison solve")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-iterations", type=int, default=REFERENCE_SAMPLE_ITERATIONS)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-LP section")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint section")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own CUDA PDHG")
    ap.add_argument("--no-qp", action="store_true", help="skip the convex-QP section")
    ap.add_argument("--profile-qp", type=int, metavar="PERIODS", default=0,
                    help="profile case: the QP on a slice of this many periods, 200 iterations")
    ap.add_argument("--no-zipf", action="store_true",
                    help="skip the load-balance stress LP (Zipf row lengths)")
    ap.add_argument("--profile-case", type=int, metavar="PERIODS", default=0,
                    help="run only the small kernel-capture case with this many periods")
    ap.add_argument("--profile-iterations", type=int, default=40)
    ap.add_argument("--profile-zipf", action="store_true",
                    help="profile case on the 500,000 x 1,000,000 Zipf-row LP")
    args = ap.parse_args()
    if args.profile_qp:
        profile_qp(args.profile_qp)
        return
    if args.profile_case or args.profile_zipf:
        profile_case(args.profile_case, args.precision, args.profile_iterations,
                     zipf=args.profile_zipf)
        return
    rank, world, local, dist = dist_setup()
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        lp = make_workload()
        values, samples = [], []
        for step in range(args.warmup + args.steps):
            timed = step >= args.warmup
            setup, per_it, _, r = cpu_reference(
                lp, REFERENCE_SAMPLE_ITERATIONS if timed else 0, threads)
            if timed:
                values.append(setup + per_it * FP64_ITERATIONS_TO_1E8)
                samples.append((setup, per_it, relative_kkt(r.residuals), r.iterations))
        value = max(values)
        setup, per_it, kkt, its = samples[values.index(value)]
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * value, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(lp, "fp64"),
                "cpu_baseline": {"value": value, "unit": "s", "cores": threads,
                                 "kind": cpu_kind()[0], "port_of": cpu_kind()[1],
                                 "host": host_cpu(),
                                 "sample": f"per timed step: {cpu_kind()[0]} setup + "
                                           f"{REFERENCE_SAMPLE_ITERATIONS} FP64 iterations on "
                                           f"{threads} threads; warm-up steps: setup only",
                                 "measured": {"setup_s": setup, "s_per_iteration": per_it,
                                              "iterations": its,
                                              "evaluation_points": its // 40,
                                              "relative_kkt_reached": kkt},
                                 "extrapolated": True,
                                 "projected_iterations": FP64_ITERATIONS_TO_1E8,
                                 "projection": "setup + s_per_iteration x the accepted "
                                               "iterations the FP64 method needs to 1e-8 on "
                                               "this LP (measured by this bench's FP64 GPU "
                                               "solve)"},
                "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from sankhya_gb300 import build, capi

    build.build_lpgen()
    build.build_engine()
    lp = make_workload()
    peak, peak_kind = peaks()
    eng = capi.PdhgEngine(local)
    eng.load(lp)
    opts = dict(tolerance=TOLERANCE, stop_rule="relative")

    for _ in range(args.warmup):
        eng.solve(precision=args.precision, **opts)
    if dist:
        dist.barrier()
    results = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            results.append(eng.solve(precision=args.precision, **opts))
    if dist:
        dist.barrier()
    step_s = max(r.device_seconds for r in results)
    last = results[-1]
    launches = sum(r.kernel_launches for r in results)
    roof = kernel_roofline(eng, lp, args.precision, peak, last.staged_fraction)

    fp64 = froof = f = None
    if args.precision != "fp64" and not args.no_fp64:
        f = eng.solve(precision="fp64", **opts)
        froof = kernel_roofline(eng, lp, "fp64", peak, f.staged_fraction)
        fp64 = {"seconds": f.device_seconds, "iterations": f.iterations, "status": f.status_name,
                "relative_kkt": relative_kkt(f.residuals),
                "objective_rel_err": abs(f.objective - lp.fstar) / max(1.0, abs(lp.fstar)),
                "us_per_attempt": 1e6 * f.loop_seconds / max(1, f.attempts),
                "speedup_of_mixed": f.device_seconds / step_s}

    # End to end through the C ABI from host buffers (page-locked where a device is there to
    # pin with): load (H2D), solve, solution (D2H). Staging the inputs in page-locked memory
    # is timed apart (pin_seconds); value_with_pinning adds it.
    t0 = time.perf_counter()
    lp_host, pinned = pinned_lp(lp)
    pin_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    eng2 = capi.PdhgEngine(local)
    eng2.load(lp_host)
    r2 = eng2.solve(precision=args.precision, **opts)
    x, d, y = eng2.solution()
    e2e_s = time.perf_counter() - t0
    eng2.close()
    h2d = (lp.col_starts.nbytes + lp.row_index.nbytes + lp.values.nbytes + lp.col_cost.nbytes
           + lp.col_lower.nbytes + lp.col_upper.nbytes + lp.row_lower.nbytes
           + lp.row_upper.nbytes)
    d2h = x.nbytes + d.nbytes + y.nbytes

    if dist:
        import torch

        t = torch.tensor([step_s, e2e_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_s, e2e_s = float(t[0]), float(t[1])
    if rank != 0:
        return

    # The further sections report an error in their own field rather than lose the line.
    batched = adjoint = zipf = None
    if not args.no_batch:
        try:
            batched = batched_section(local)
        except Exception as exc:  # noqa: BLE001
            batched = {"error": f"{type(exc).__name__}: {exc}"}
    if not args.no_adjoint:
        try:
            adjoint = adjoint_section(local)
        except Exception as exc:  # noqa: BLE001
            adjoint = {"error": f"{type(exc).__name__}: {exc}"}
    if not args.no_zipf:
        try:
            zipf = zipf_section(local, peak)
        except Exception as exc:  # noqa: BLE001
            zipf = {"error": f"{type(exc).__name__}: {exc}"}
    qp = None
    if not args.no_qp:
        try:
            qp = qp_section(local, peak, lp, cpu=not args.no_cpu_baseline)
        except Exception as exc:  # noqa: BLE001
            qp = {"error": f"{type(exc).__name__}: {exc}"}

    cpu = None
    if not args.no_cpu_baseline:
        its = f.iterations if f is not None else FP64_ITERATIONS_TO_1E8
        its_from = ("the FP64 GPU solve of this run" if f is not None
                    else "the FP64 iteration count measured by an earlier run of this bench")
        setup, per_it, sample_s, sr = cpu_reference(lp, args.cpu_iterations, threads)
        try:
            setup1, per_it1, sample1, _ = cpu_reference(lp, max(2, args.cpu_iterations // 4), 1)
            single = {"value": setup1 + per_it1 * its, "unit": "s", "cores": 1,
                      "setup_s": setup1, "s_per_iteration": per_it1, "sample_s": sample1}
        except Exception as exc:  # noqa: BLE001
            single = {"error": f"{type(exc).__name__}: {exc}"}
        try:
            limited = cpu_time_limited(lp, threads, CPU_TIME_LIMIT)
        except Exception as exc:  # noqa: BLE001
            limited = {"error": f"{type(exc).__name__}: {exc}"}
        cpu = {"value": setup + per_it * its, "unit": "s", "cores": threads,
               "kind": cpu_kind()[0], "port_of": cpu_kind()[1], "host": host_cpu(),
               "sample": f"{cpu_kind()[0]} setup + {args.cpu_iterations} FP64 iterations on {threads} "
                         f"threads ({sample_s:.1f} s of CPU work), extrapolated to {its} "
                         f"iterations ({its_from})",
               "extrapolated": True, "setup_s": setup, "s_per_iteration": per_it,
               "sample_relative_kkt": relative_kkt(sr.residuals) if sr is not None else None,
               "time_limited_run": limited, "single_thread": single}

    reference_gpu = None
    if not args.no_reference_gpu:
        try:
            reference_gpu = reference_gpu_section()
        except Exception as exc:  # noqa: BLE001
            reference_gpu = {"error": f"{type(exc).__name__}: {exc}"}

    dominant = "k_dual" if roof["k_dual_ms"] >= roof["k_primal_ms"] else "k_primal"
    kname = {"k_dual": "row pass (A xbar, A dx, dual update)",
             "k_primal": "column pass (A^T y, primal update)"}[dominant]
    suffix = "_f" if args.precision == "mixed" else ""
    traffic = ncu_traffic().get(dominant + suffix)
    parity = parity_object(lp, last, f, step_s, f.device_seconds if f is not None else None)
    # The nested sections come first and the contract keys and the compact summaries last:
    # a reader that keeps only the end of the line still has the parity verdict.
    line = {
        "spmv_gbs": roof, "fp64_kernels": froof, "batched": batched, "adjoint": adjoint,
        "zipf": zipf, "qp": qp, "reference_gpu": reference_gpu,
        "metric": METRIC, "value": step_s, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded planted-optimum generator)",
        "config": workload_config(lp, args.precision),
        "status": last.status_name, "iterations": last.iterations, "attempts": last.attempts,
        "refinement_rounds": last.refinements, "restarts": last.restarts,
        "setup_s": last.setup_seconds, "loop_s": last.loop_seconds,
        "us_per_attempt": 1e6 * last.loop_seconds / max(1, last.attempts),
        "lps_per_s": world / step_s,
        "roofline": {"bound": "hbm", "kernel": f"{dominant}{suffix}: {kname}",
                     "achieved": roof[dominant + "_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": roof[dominant + "_gbs"] / peak, "traffic": traffic,
                     "algorithmic_bytes": roof[dominant + "_bytes"],
                     "peak_source": peak_kind},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "status": r2.status_name, "pinned_inputs": pinned,
                "pin_seconds": pin_s, "value_with_pinning": e2e_s + pin_s},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "fp64": fp64,
        "parity": parity,
    }
    print(json.dumps(line))
    if parity is not None and not parity["same_answer"]:
        sys.exit(3)


if __name__ == "__main__":
    main()

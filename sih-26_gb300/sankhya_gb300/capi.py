"""ctypes binding of include/sankhya_gb300.h (lib/libsankhya_gb300.so).

There is no CPU fallback: if the library is missing or no GPU is usable, every call raises
``EngineError``. ``solve_pdhg_gpu(lp, options)`` mirrors the reference seam
``sankhya::gpu::solve_pdhg_gpu(model, options, logger, control)`` (src/gpu/pdhg_gpu.hpp:19)
and takes the reference's option names (src/util/options.cpp): ``pdhg_tolerance``,
``iteration_limit``, ``time_limit``, ``pdhg_restart``, ``pdhg_stop_at_request``,
``random_seed``, plus the engine's ``pdhg_precision`` ("fp64" | "mixed") and
``pdhg_stop_rule`` ("standard" | "relative").
"""
from __future__ import annotations

import ctypes
import os
import threading
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from . import _paths
from .model import LP

OK = 0
STATUS_NAMES = {0: "not_solved", 1: "optimal", 2: "feasible", 3: "infeasible",
                5: "iteration_limit", 6: "time_limit", 8: "numerical_error", 9: "model_error",
                11: "interrupted"}
PRECISIONS = {"fp64": 0, "mixed": 1}
STOP_RULES = {"standard": 0, "relative": 1}

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double,
                          ctypes.c_double, ctypes.c_double, ctypes.c_double)
POLL_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double)


class EngineError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class CLp(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("col_starts", _I),
                ("row_index", _I), ("values", _D), ("col_cost", _D), ("col_lower", _D),
                ("col_upper", _D), ("row_lower", _D), ("row_upper", _D),
                ("sense", ctypes.c_double), ("objective_offset", ctypes.c_double)]


class CParams(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("iteration_limit", ctypes.c_int64),
                ("time_limit", ctypes.c_double), ("restart", ctypes.c_int32),
                ("stop_at_request", ctypes.c_int32), ("random_seed", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("steps_per_poll", ctypes.c_int32),
                ("stop_rule", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("interrupt", ctypes.POINTER(ctypes.c_int32)), ("log", LOG_FN),
                ("log_user", ctypes.c_void_p), ("poll", POLL_FN), ("poll_user", ctypes.c_void_p)]


class CResiduals(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "primal", "dual", "gap", "primal_objective", "dual_objective", "absolute_primal",
        "absolute_dual", "gap_as_verified", "complementarity")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("iterations", ctypes.c_int64), ("attempts", ctypes.c_int64),
                ("restarts", ctypes.c_int64), ("evaluations", ctypes.c_int64),
                ("refinements", ctypes.c_int64), ("objective", ctypes.c_double),
                ("dual_bound", ctypes.c_double), ("final_residuals", CResiduals),
                ("spectral_norm", ctypes.c_double), ("scaled_min_abs", ctypes.c_double),
                ("scaled_max_abs", ctypes.c_double), ("setup_seconds", ctypes.c_double),
                ("loop_seconds", ctypes.c_double), ("solve_seconds", ctypes.c_double),
                ("device_seconds", ctypes.c_double), ("kernel_launches", ctypes.c_int64),
                ("staged_fraction", ctypes.c_double * 2),
                ("message", ctypes.c_char * 512)]


class CAdjointInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("basic_cols", ctypes.c_int32),
                ("active_rows", ctypes.c_int32), ("iterations", ctypes.c_int32 * 2),
                ("residual", ctypes.c_double * 2)]


class CBatchItem(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("iterations", ctypes.c_int64), ("attempts", ctypes.c_int64),
                ("restarts", ctypes.c_int64), ("evaluations", ctypes.c_int64),
                ("objective", ctypes.c_double), ("dual_bound", ctypes.c_double),
                ("final_residuals", CResiduals), ("spectral_norm", ctypes.c_double),
                ("farkas_value", ctypes.c_double), ("refinements", ctypes.c_int64)]


class CQpProblem(ctypes.Structure):
    _fields_ = [("lp", CLp), ("hessian_starts", _I), ("hessian_index", _I),
                ("hessian_values", _D)]


class CQpParams(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("iteration_limit", ctypes.c_int64),
                ("time_limit", ctypes.c_double), ("random_seed", ctypes.c_int64),
                ("periods_per_poll", ctypes.c_int32), ("column_lanes", ctypes.c_int32),
                ("row_lanes", ctypes.c_int32), ("staging", ctypes.c_int32),
                ("interrupt", ctypes.POINTER(ctypes.c_int32)), ("log", LOG_FN),
                ("log_user", ctypes.c_void_p), ("poll", POLL_FN),
                ("poll_user", ctypes.c_void_p)]


class CQpResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("ceiling", ctypes.c_int32),
                ("iterations", ctypes.c_int64)] + [(k, ctypes.c_double) for k in (
                    "primal_residual", "dual_residual", "norm_a", "norm_q", "tau", "sigma",
                    "objective", "setup_seconds", "loop_seconds", "solve_seconds",
                    "device_seconds")] + [
                ("kernel_launches", ctypes.c_int64), ("column_lanes", ctypes.c_int32),
                ("row_lanes", ctypes.c_int32), ("message", ctypes.c_char * 256)]


EXPORTS = [
    "sankhya_gb300_last_error", "sankhya_gb300_device_available",
    "sankhya_gb300_device_free_memory", "sankhya_gb300_device_compute_capability",
    "sankhya_gb300_estimate_memory", "sankhya_gb300_pdhg_create", "sankhya_gb300_pdhg_destroy",
    "sankhya_gb300_pdhg_load", "sankhya_gb300_pdhg_solve", "sankhya_gb300_pdhg_solution",
    "sankhya_gb300_pdhg_scaling", "sankhya_gb300_pdhg_spmv", "sankhya_gb300_pdhg_time_kernels",
    "sankhya_gb300_pdhg_spmv_noalloc", "sankhya_gb300_batch_create",
    "sankhya_gb300_batch_destroy", "sankhya_gb300_batch_load", "sankhya_gb300_batch_solve",
    "sankhya_gb300_batch_solution", "sankhya_gb300_batch_adjoint", "sankhya_gb300_batch_polish",
    "sankhya_gb300_batch_schedule", "sankhya_gb300_batch_last_schedule",
    "sankhya_gb300_batch_ray", "sankhya_gb300_batch_set_point",
    "sankhya_gb300_qp_create", "sankhya_gb300_qp_destroy", "sankhya_gb300_qp_load",
    "sankhya_gb300_qp_solve", "sankhya_gb300_qp_solution", "sankhya_gb300_qp_time_kernels",
]

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _paths.ENGINE_LIB


def load_library():
    """Load the engine library (raises if it is not built: there is no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_paths.ENGINE_LIB):
            raise EngineError(7, f"{_paths.ENGINE_LIB} is not built; run __graft_entry__.build()")
        lib = ctypes.CDLL(_paths.ENGINE_LIB)
        lib.sankhya_gb300_last_error.restype = ctypes.c_char_p
        lib.sankhya_gb300_last_error.argtypes = []
        lib.sankhya_gb300_device_available.argtypes = [ctypes.c_char_p, ctypes.c_int32]
        lib.sankhya_gb300_device_free_memory.argtypes = [ctypes.POINTER(ctypes.c_size_t)] * 2
        lib.sankhya_gb300_device_compute_capability.argtypes = [ctypes.POINTER(ctypes.c_int32)] * 2
        lib.sankhya_gb300_estimate_memory.argtypes = [ctypes.c_int32, ctypes.c_int32,
                                                      ctypes.c_int64, ctypes.c_int32]
        lib.sankhya_gb300_estimate_memory.restype = ctypes.c_size_t
        lib.sankhya_gb300_pdhg_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
        lib.sankhya_gb300_pdhg_destroy.argtypes = [ctypes.c_void_p]
        lib.sankhya_gb300_pdhg_load.argtypes = [ctypes.c_void_p, ctypes.POINTER(CLp)]
        lib.sankhya_gb300_pdhg_solve.argtypes = [ctypes.c_void_p, ctypes.POINTER(CParams),
                                                 ctypes.POINTER(CResult)]
        lib.sankhya_gb300_pdhg_solution.argtypes = [ctypes.c_void_p, _D, _D, _D]
        lib.sankhya_gb300_pdhg_scaling.argtypes = [ctypes.c_void_p, ctypes.c_int64, _D, _D, _D, _D]
        lib.sankhya_gb300_pdhg_spmv.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                                _D, _D]
        lib.sankhya_gb300_pdhg_time_kernels.argtypes = [ctypes.c_void_p, ctypes.c_int32, _D]
        lib.sankhya_gb300_batch_create.argtypes = [ctypes.c_int32,
                                                   ctypes.POINTER(ctypes.c_void_p)]
        lib.sankhya_gb300_batch_destroy.argtypes = [ctypes.c_void_p]
        lib.sankhya_gb300_batch_load.argtypes = [ctypes.c_void_p, ctypes.c_int32,
                                                 ctypes.POINTER(CLp)]
        lib.sankhya_gb300_batch_solve.argtypes = [ctypes.c_void_p, ctypes.POINTER(CParams),
                                                  ctypes.POINTER(CBatchItem), _D]
        lib.sankhya_gb300_batch_solution.argtypes = [ctypes.c_void_p, ctypes.c_int32, _D, _D,
                                                     _D]
        lib.sankhya_gb300_batch_ray.argtypes = [ctypes.c_void_p, ctypes.c_int32, _D]
        lib.sankhya_gb300_batch_set_point.argtypes = [ctypes.c_void_p, ctypes.c_int32, _D, _D,
                                                      _D]
        lib.sankhya_gb300_batch_schedule.argtypes = [ctypes.c_void_p, ctypes.c_int32,
                                                     ctypes.c_int32]
        lib.sankhya_gb300_batch_last_schedule.argtypes = [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), _D]
        _PP = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))
        lib.sankhya_gb300_batch_adjoint.argtypes = [ctypes.c_void_p, _PP, _PP, _D, _PP, _PP, _PP,
                                                    _PP, _PP, ctypes.POINTER(CAdjointInfo)]
        lib.sankhya_gb300_batch_polish.argtypes = [ctypes.c_void_p, ctypes.POINTER(CBatchItem),
                                                   ctypes.POINTER(CAdjointInfo)]
        lib.sankhya_gb300_pdhg_spmv_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int32,
                                                        ctypes.c_int32, ctypes.c_void_p,
                                                        ctypes.c_void_p, ctypes.c_void_p]
        lib.sankhya_gb300_qp_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
        lib.sankhya_gb300_qp_destroy.argtypes = [ctypes.c_void_p]
        lib.sankhya_gb300_qp_load.argtypes = [ctypes.c_void_p, ctypes.POINTER(CQpProblem)]
        lib.sankhya_gb300_qp_solve.argtypes = [ctypes.c_void_p, ctypes.POINTER(CQpParams),
                                               ctypes.POINTER(CQpResult)]
        lib.sankhya_gb300_qp_solution.argtypes = [ctypes.c_void_p, _D, _D, _D]
        lib.sankhya_gb300_qp_time_kernels.argtypes = [ctypes.c_void_p, ctypes.c_int32, _D]
        for name in EXPORTS:
            if name not in ("sankhya_gb300_last_error", "sankhya_gb300_estimate_memory"):
                getattr(lib, name).restype = ctypes.c_int
        _lib = lib
        return lib


def _check(code: int):
    if code != OK:
        msg = load_library().sankhya_gb300_last_error().decode(errors="replace")
        raise EngineError(code, msg)


def _ptr(a, ctype=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def device_available() -> tuple[bool, str]:
    lib = load_library()
    buf = ctypes.create_string_buffer(256)
    ok = lib.sankhya_gb300_device_available(buf, 256) == OK
    return ok, buf.value.decode(errors="replace")


def estimate_memory(rows: int, cols: int, nnz: int, precision: str = "fp64") -> int:
    return int(load_library().sankhya_gb300_estimate_memory(rows, cols, nnz,
                                                            PRECISIONS[precision]))


@dataclass
class Result:
    status: int
    status_name: str
    converged: bool
    iterations: int
    attempts: int
    restarts: int
    evaluations: int
    refinements: int
    objective: float
    dual_bound: float
    residuals: dict
    spectral_norm: float
    scaled_min_abs: float
    scaled_max_abs: float
    setup_seconds: float
    loop_seconds: float
    solve_seconds: float
    device_seconds: float
    kernel_launches: int
    staged_fraction: tuple
    message: str


class PdhgEngine:
    """One engine on one device: load an LP once, solve it any number of times."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.sankhya_gb300_pdhg_create(device, ctypes.byref(h)))
        self._h = h
        self._lp: Optional[LP] = None

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sankhya_gb300_pdhg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def load(self, lp: LP):
        lp = lp.contiguous()
        c = CLp(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                _ptr(lp.row_index, ctypes.c_int32), _ptr(lp.values), _ptr(lp.col_cost),
                _ptr(lp.col_lower), _ptr(lp.col_upper), _ptr(lp.row_lower), _ptr(lp.row_upper),
                lp.sense, lp.objective_offset)
        _check(self._lib.sankhya_gb300_pdhg_load(self._h, ctypes.byref(c)))
        self._lp = lp

    def solve(self, tolerance: float = 1e-4, iteration_limit: int = -1,
              time_limit: Optional[float] = None, restart: bool = True,
              stop_at_request: bool = False, random_seed: int = 0, precision: str = "fp64",
              steps_per_poll: int = 0, interrupt: Optional[np.ndarray] = None,
              log: Optional[Callable] = None, stop_rule: str = "standard",
              poll: Optional[Callable] = None) -> Result:
        """``poll(iteration, objective) -> bool`` is asked at every status snapshot; True
        interrupts the solve."""
        cb = LOG_FN(lambda user, it, obj, p, d, s: log(it, obj, p, d, s)) if log else LOG_FN()
        pcb = POLL_FN(lambda user, it, obj: int(bool(poll(it, obj)))) if poll else POLL_FN()
        intr = (interrupt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
                if interrupt is not None else ctypes.POINTER(ctypes.c_int32)())
        params = CParams(tolerance, iteration_limit,
                         1e308 if time_limit is None else float(time_limit), int(restart),
                         int(stop_at_request), random_seed, PRECISIONS[precision],
                         steps_per_poll, STOP_RULES[stop_rule], 0, intr, cb, None, pcb, None)
        r = CResult()
        _check(self._lib.sankhya_gb300_pdhg_solve(self._h, ctypes.byref(params), ctypes.byref(r)))
        return Result(r.status, STATUS_NAMES.get(r.status, str(r.status)), bool(r.converged),
                      r.iterations, r.attempts, r.restarts, r.evaluations, r.refinements,
                      r.objective, r.dual_bound, r.final_residuals.as_dict(), r.spectral_norm,
                      r.scaled_min_abs, r.scaled_max_abs, r.setup_seconds, r.loop_seconds,
                      r.solve_seconds, r.device_seconds, r.kernel_launches,
                      (r.staged_fraction[0], r.staged_fraction[1]),
                      r.message.decode(errors="replace"))

    def time_kernels(self, reps: int = 20):
        """Mean device milliseconds of the primal and the dual pass (CUDA events on the
        engine's stream), measured on the state of the last solve."""
        ms = np.zeros(2)
        _check(self._lib.sankhya_gb300_pdhg_time_kernels(self._h, reps, _ptr(ms)))
        return float(ms[0]), float(ms[1])

    def solution(self):
        lp = self._lp
        x = np.zeros(lp.cols)
        d = np.zeros(lp.cols)
        y = np.zeros(lp.rows)
        _check(self._lib.sankhya_gb300_pdhg_solution(self._h, _ptr(x), _ptr(d), _ptr(y)))
        return x, d, y

    def scaling(self, random_seed: int = 0):
        lp = self._lp
        dr = np.zeros(lp.rows)
        dc = np.zeros(lp.cols)
        vals = np.zeros(lp.nnz)
        norm = ctypes.c_double()
        _check(self._lib.sankhya_gb300_pdhg_scaling(self._h, random_seed, _ptr(dr), _ptr(dc),
                                                    _ptr(vals), ctypes.byref(norm)))
        return dr, dc, vals, norm.value

    def spmv(self, op: int, vec, scaled: bool = False):
        lp = self._lp
        vec = np.ascontiguousarray(vec, dtype=np.float64)
        out = np.zeros(lp.rows if op == 0 else lp.cols)
        _check(self._lib.sankhya_gb300_pdhg_spmv(self._h, op, int(scaled), _ptr(vec), _ptr(out)))
        return out

    def spmv_device(self, op: int, device_in: int, device_out: int, scaled: bool = False,
                    stream: Optional[int] = None):
        """The product on caller-owned device buffers (raw device addresses), enqueued on
        `stream` (a cudaStream_t handle; None = the engine's stream); allocates nothing and
        does not wait for the work."""
        _check(self._lib.sankhya_gb300_pdhg_spmv_noalloc(
            self._h, op, int(scaled), ctypes.c_void_p(device_in), ctypes.c_void_p(device_out),
            ctypes.c_void_p(stream) if stream else None))


@dataclass
class QpResult:
    status: int
    status_name: str
    ceiling: bool
    iterations: int
    primal_residual: float
    dual_residual: float
    norm_a: float
    norm_q: float
    tau: float
    sigma: float
    objective: float
    setup_seconds: float
    loop_seconds: float
    solve_seconds: float
    device_seconds: float
    kernel_launches: int
    column_lanes: int
    row_lanes: int
    message: str


class QpEngine:
    """The convex-QP engine (Condat-Vu, src/qp/qp_condat_vu.cpp) on one device: load a QP
    once, solve it any number of times. The caller owns the convexity decision beyond the
    engine's diagonal test (the seam runs the reference's check_convexity first)."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.sankhya_gb300_qp_create(device, ctypes.byref(h)))
        self._h = h
        self._qp = None

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sankhya_gb300_qp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def load(self, qp):
        qp = qp.contiguous()
        lp = qp.lp
        c = CLp(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                _ptr(lp.row_index, ctypes.c_int32), _ptr(lp.values), _ptr(lp.col_cost),
                _ptr(lp.col_lower), _ptr(lp.col_upper), _ptr(lp.row_lower), _ptr(lp.row_upper),
                lp.sense, lp.objective_offset)
        p = CQpProblem(c, _ptr(qp.hessian_starts, ctypes.c_int32),
                       _ptr(qp.hessian_index, ctypes.c_int32), _ptr(qp.hessian_values))
        _check(self._lib.sankhya_gb300_qp_load(self._h, ctypes.byref(p)))
        self._qp = qp

    def solve(self, tolerance: float = 1e-8, iteration_limit: int = -1,
              time_limit: Optional[float] = None, random_seed: int = 0,
              periods_per_poll: int = 0, column_lanes: int = 0, row_lanes: int = 0,
              interrupt: Optional[np.ndarray] = None, log: Optional[Callable] = None,
              poll: Optional[Callable] = None, staging: bool = False) -> QpResult:
        cb = LOG_FN(lambda user, it, obj, p, d, s: log(it, obj, p, d, s)) if log else LOG_FN()
        pcb = POLL_FN(lambda user, it, obj: int(bool(poll(it, obj)))) if poll else POLL_FN()
        intr = (interrupt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
                if interrupt is not None else ctypes.POINTER(ctypes.c_int32)())
        params = CQpParams(tolerance, iteration_limit,
                           1e308 if time_limit is None else float(time_limit), random_seed,
                           periods_per_poll, column_lanes, row_lanes, int(bool(staging)),
                           intr, cb, None, pcb, None)
        r = CQpResult()
        _check(self._lib.sankhya_gb300_qp_solve(self._h, ctypes.byref(params), ctypes.byref(r)))
        return QpResult(r.status, STATUS_NAMES.get(r.status, str(r.status)), bool(r.ceiling),
                        r.iterations, r.primal_residual, r.dual_residual, r.norm_a, r.norm_q,
                        r.tau, r.sigma, r.objective, r.setup_seconds, r.loop_seconds,
                        r.solve_seconds, r.device_seconds, r.kernel_launches, r.column_lanes,
                        r.row_lanes, r.message.decode(errors="replace"))

    def solution(self):
        """(col_value, col_dual, row_dual) as solve_convex_qp fills Solution."""
        qp = self._qp
        x = np.zeros(qp.cols)
        d = np.zeros(qp.cols)
        y = np.zeros(qp.rows)
        _check(self._lib.sankhya_gb300_qp_solution(self._h, _ptr(x), _ptr(d), _ptr(y)))
        return x, d, y

    def time_kernels(self, reps: int = 20):
        """Mean device milliseconds of the column and the row pass on the last solve's state."""
        ms = np.zeros(2)
        _check(self._lib.sankhya_gb300_qp_time_kernels(self._h, reps, _ptr(ms)))
        return float(ms[0]), float(ms[1])


@dataclass
class BatchItem:
    status: int
    status_name: str
    converged: bool
    iterations: int
    attempts: int
    restarts: int
    evaluations: int
    objective: float
    dual_bound: float
    residuals: dict
    spectral_norm: float
    farkas_value: float
    refinements: int = 0


class BatchEngine:
    """Many LPs solved together, one thread block per LP (sankhya_gb300_batch_*). LPs whose
    matrix arrays are the same numpy objects share one device copy of the matrix."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.sankhya_gb300_batch_create(device, ctypes.byref(h)))
        self._h = h
        self._lps = []
        self._keep = None

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sankhya_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def load(self, lps):
        lps = [lp.contiguous() for lp in lps]
        arr = (CLp * len(lps))()
        for k, lp in enumerate(lps):
            arr[k] = CLp(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                         _ptr(lp.row_index, ctypes.c_int32), _ptr(lp.values), _ptr(lp.col_cost),
                         _ptr(lp.col_lower), _ptr(lp.col_upper), _ptr(lp.row_lower),
                         _ptr(lp.row_upper), lp.sense, lp.objective_offset)
        _check(self._lib.sankhya_gb300_batch_load(self._h, len(lps), arr))
        self._lps = lps

    def solve(self, tolerance: float = 1e-4, iteration_limit: int = -1, restart: bool = True,
              stop_at_request: bool = False, random_seed: int = 0,
              stop_rule: str = "standard", precision: str = "fp64"):
        """Returns ([BatchItem] in load order, device seconds of the solve)."""
        params = CParams(tolerance, iteration_limit, 1e308, int(restart), int(stop_at_request),
                         random_seed, PRECISIONS[precision], 0, STOP_RULES[stop_rule], 0,
                         ctypes.POINTER(ctypes.c_int32)(), LOG_FN(), None, POLL_FN(), None)
        items = (CBatchItem * len(self._lps))()
        sec = np.zeros(1)
        _check(self._lib.sankhya_gb300_batch_solve(self._h, ctypes.byref(params), items,
                                                   _ptr(sec)))
        out = []
        for it in items:
            out.append(BatchItem(it.status, STATUS_NAMES.get(it.status, str(it.status)),
                                 bool(it.converged), it.iterations, it.attempts, it.restarts,
                                 it.evaluations, it.objective, it.dual_bound,
                                 it.final_residuals.as_dict(), it.spectral_norm,
                                 it.farkas_value, it.refinements))
        return out, float(sec[0])

    def set_schedule(self, lanes: int = 0, threads: int = 0):
        """The schedule of the next solves: lanes per row or column and threads per LP;
        0, 0 (the default) autotunes every solve (sankhya_gb300_batch_schedule)."""
        _check(self._lib.sankhya_gb300_batch_schedule(self._h, lanes, threads))

    def last_schedule(self):
        """(lanes, threads, autotuning seconds) of the last solve."""
        lanes, threads = ctypes.c_int32(), ctypes.c_int32()
        sec = np.zeros(1)
        _check(self._lib.sankhya_gb300_batch_last_schedule(self._h, ctypes.byref(lanes),
                                                           ctypes.byref(threads), _ptr(sec)))
        return int(lanes.value), int(threads.value), float(sec[0])

    def ray(self, index: int):
        """The dual direction LP `index` was reported infeasible by (sankhya_gb300_batch_ray);
        certify.farkas_share checks it."""
        y = np.zeros(self._lps[index].rows)
        _check(self._lib.sankhya_gb300_batch_ray(self._h, index, _ptr(y)))
        return y

    def set_point(self, index: int, col_value, col_dual, row_dual):
        """Replace LP `index`'s reported point (as solution() returns it): the polish's warm
        start (sankhya_gb300_batch_set_point)."""
        lp = self._lps[index]
        x = np.ascontiguousarray(col_value, dtype=np.float64)
        d = np.ascontiguousarray(col_dual, dtype=np.float64)
        y = np.ascontiguousarray(row_dual, dtype=np.float64)
        if x.shape != (lp.cols,) or d.shape != (lp.cols,) or y.shape != (lp.rows,):
            raise ValueError("a point of the LP's shape is expected")
        _check(self._lib.sankhya_gb300_batch_set_point(self._h, index, _ptr(x), _ptr(d),
                                                       _ptr(y)))

    def solution(self, index: int):
        lp = self._lps[index]
        x = np.zeros(lp.cols)
        d = np.zeros(lp.cols)
        y = np.zeros(lp.rows)
        _check(self._lib.sankhya_gb300_batch_solution(self._h, index, _ptr(x), _ptr(d), _ptr(y)))
        return x, d, y

    def polish(self):
        """Active-set polish of the last solve (sankhya_gb300_batch_polish). Returns
        ([BatchItem] with the polished statuses / objectives / residuals, [info dict])."""
        n = len(self._lps)
        items = (CBatchItem * n)()
        info = (CAdjointInfo * n)()
        _check(self._lib.sankhya_gb300_batch_polish(self._h, items, info))
        out = [BatchItem(it.status, STATUS_NAMES.get(it.status, str(it.status)), True, 0, 0, 0,
                         0, it.objective, it.dual_bound, it.final_residuals.as_dict(), 0.0, 0.0)
               for it in items]
        return out, [dict(status=i.status, basic_cols=i.basic_cols, active_rows=i.active_rows,
                          iterations=tuple(i.iterations), residual=tuple(i.residual))
                     for i in info]

    def adjoint(self, dl_dx=None, dl_dy=None, dl_df=None):
        """Gradients through the last solve (sankhya_gb300_batch_adjoint). dl_dx / dl_dy are
        lists (one array per LP, or None) of upstream gradients with respect to col_value and
        row_dual; dl_df a sequence of upstream gradients with respect to the objective.
        Returns a list of dicts with dc, drl, dru, dl, du and the solve info."""
        n = len(self._lps)
        keep = []

        def ins(arrs, size_of):
            ptrs = (ctypes.POINTER(ctypes.c_double) * n)()
            for k in range(n):
                a = None if arrs is None else arrs[k]
                if a is not None:
                    a = np.ascontiguousarray(a, dtype=np.float64)
                    assert a.shape == (size_of(self._lps[k]),)
                    keep.append(a)
                    ptrs[k] = _ptr(a)
            return ptrs

        def outs(size_of):
            arrs = [np.zeros(size_of(lp)) for lp in self._lps]
            ptrs = (ctypes.POINTER(ctypes.c_double) * n)(*[_ptr(a) for a in arrs])
            return arrs, ptrs

        px = ins(dl_dx, lambda lp: lp.cols)
        py = ins(dl_dy, lambda lp: lp.rows)
        gf = np.zeros(n) if dl_df is None else np.ascontiguousarray(dl_df, dtype=np.float64)
        dc, pdc = outs(lambda lp: lp.cols)
        dl, pdl = outs(lambda lp: lp.cols)
        du, pdu = outs(lambda lp: lp.cols)
        drl, pdrl = outs(lambda lp: lp.rows)
        dru, pdru = outs(lambda lp: lp.rows)
        info = (CAdjointInfo * n)()
        _check(self._lib.sankhya_gb300_batch_adjoint(self._h, px, py, _ptr(gf), pdc, pdrl, pdru,
                                                     pdl, pdu, info))
        return [dict(dc=dc[k], drl=drl[k], dru=dru[k], dl=dl[k], du=du[k],
                     status=info[k].status, basic_cols=info[k].basic_cols,
                     active_rows=info[k].active_rows,
                     iterations=tuple(info[k].iterations), residual=tuple(info[k].residual))
                for k in range(n)]


@dataclass
class Solution:
    """The fields of sankhya::Solution that solve_pdhg fills (src/pdhg/pdhg.cpp:487-558)."""
    status: str
    objective: float
    dual_bound: float
    col_value: np.ndarray
    col_dual: np.ndarray
    row_dual: np.ndarray
    iterations: int
    message: str
    algorithm: str = "pdhg-gpu"
    result: Optional[Result] = None
    extra: dict = field(default_factory=dict)


def solve_pdhg_gpu(lp: LP, options: Optional[dict] = None, device: int = 0,
                   engine: Optional[PdhgEngine] = None, log: Optional[Callable] = None,
                   interrupt: Optional[np.ndarray] = None) -> Solution:
    """The GPU PDHG behind the reference seam's contract: never falls back to the CPU; a
    model defect is status "model_error", a device failure raises EngineError."""
    o = {"pdhg_tolerance": 1e-4, "iteration_limit": -1, "time_limit": None,
         "pdhg_restart": True, "pdhg_stop_at_request": False, "random_seed": 0,
         "pdhg_precision": "fp64", "pdhg_stop_rule": "standard", "steps_per_poll": 0}
    o.update(options or {})
    own = engine is None
    eng = engine or PdhgEngine(device)
    try:
        try:
            eng.load(lp)
        except EngineError as e:
            if e.code == 3:
                z = np.zeros
                return Solution("model_error", 0.0, float("nan"), z(lp.cols), z(lp.cols),
                                z(lp.rows), 0, str(e))
            raise
        r = eng.solve(tolerance=o["pdhg_tolerance"], iteration_limit=o["iteration_limit"],
                      time_limit=o["time_limit"], restart=o["pdhg_restart"],
                      stop_at_request=o["pdhg_stop_at_request"], random_seed=o["random_seed"],
                      precision=o["pdhg_precision"], steps_per_poll=o["steps_per_poll"],
                      interrupt=interrupt, log=log, stop_rule=o["pdhg_stop_rule"])
        x, d, y = eng.solution()
        return Solution(r.status_name, r.objective, r.dual_bound, x, d, y, r.iterations,
                        r.message, "pdhg-gpu", r)
    finally:
        if own:
            eng.close()


def solve_convex_qp_gpu(qp, options: Optional[dict] = None, device: int = 0,
                        engine: Optional["QpEngine"] = None, log: Optional[Callable] = None,
                        interrupt: Optional[np.ndarray] = None) -> Solution:
    """The GPU convex-QP engine behind sankhya::qp::solve_convex_qp's contract
    (include/sankhya/qp.hpp:20, src/qp/qp_condat_vu.cpp:164-362), with the option registry's
    names and defaults (src/util/options.cpp: qp_tolerance 1e-8, iteration_limit -1, no time
    limit, random_seed 0). Never falls back to the CPU: a model defect (the engine's own
    checks, its diagonal convexity test included) is status "model_error", a device failure
    raises EngineError. The full convexity decision is the caller's (SANKHYA's seam runs the
    reference's check_convexity). col_dual = c + Qx + sense A'y and row_dual = -sense y, as
    the reference fills them; dual_bound is the objective only when optimal."""
    o = {"qp_tolerance": 1e-8, "iteration_limit": -1, "time_limit": None, "random_seed": 0}
    o.update(options or {})
    own = engine is None
    eng = engine or QpEngine(device)
    try:
        try:
            eng.load(qp)
        except EngineError as e:
            if e.code == 3:
                z = np.zeros
                return Solution("model_error", 0.0, float("nan"), z(qp.cols), z(qp.cols),
                                z(qp.rows), 0, str(e), "qp-condat-vu-gpu")
            raise
        r = eng.solve(tolerance=o["qp_tolerance"], iteration_limit=o["iteration_limit"],
                      time_limit=o["time_limit"], random_seed=o["random_seed"],
                      interrupt=interrupt, log=log)
        x, d, y = eng.solution()
        bound = (r.objective if r.status_name == "optimal"
                 else (np.inf if qp.lp.sense < 0 else -np.inf))
        return Solution(r.status_name, r.objective, bound, x, d, y, r.iterations, r.message,
                        "qp-condat-vu-gpu", r)
    finally:
        if own:
            eng.close()

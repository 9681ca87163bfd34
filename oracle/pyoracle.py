"""ctypes binding of the checker libraries (TEST INFRASTRUCTURE ONLY).

``Oracle()`` loads oracle/liboracle.so, the C restatements of the reference PDHG and of its
convex-QP engine;
``Oracle(reference=True)`` loads oracle/_ref/libsankhya_ref.so, the reference's own sources
compiled by ``make -C oracle ref`` (only where the reference tree exists). Both expose the
same calls, so a test can run them side by side. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module; the GPU engine never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsankhya_ref.so")
# The reference checkout: SANKHYA_REFERENCE_TREE, else a `reference` directory beside this
# checkout. Where neither exists the reference checkers are not built and their tests skip.
REFERENCE_TREE = os.environ.get(
    "SANKHYA_REFERENCE_TREE",
    os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))
# A copy of the reference files the checkers are built from (`make -C oracle stage`), made
# where the reference tree exists, in the git-ignored _ref/ tree, for machines without it.
STAGE_TREE = os.path.join(HERE, "_ref", "stage")
REF_GPU_LIB = os.path.join(HERE, "_ref", "libsankhya_ref_gpu.so")

STATUS_NAMES = {0: "not_solved", 1: "optimal", 2: "feasible", 3: "infeasible",
                5: "iteration_limit", 6: "time_limit", 8: "numerical_error", 9: "model_error",
                11: "interrupted"}

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)


class CLp(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("col_starts", _I),
                ("row_index", _I), ("values", _D), ("col_cost", _D), ("col_lower", _D),
                ("col_upper", _D), ("row_lower", _D), ("row_upper", _D),
                ("sense", ctypes.c_double), ("objective_offset", ctypes.c_double)]


class CParams(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("iteration_limit", ctypes.c_int64),
                ("time_limit", ctypes.c_double), ("restart", ctypes.c_int32),
                ("stop_at_request", ctypes.c_int32), ("random_seed", ctypes.c_int64)]


class CResiduals(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "primal", "dual", "gap", "primal_objective", "dual_objective", "absolute_primal",
        "absolute_dual", "gap_as_verified", "complementarity")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("iterations", ctypes.c_int64), ("restarts", ctypes.c_int64),
                ("objective", ctypes.c_double), ("dual_bound", ctypes.c_double),
                ("final_residuals", CResiduals), ("spectral_norm", ctypes.c_double),
                ("scaled_min_abs", ctypes.c_double), ("scaled_max_abs", ctypes.c_double),
                ("solve_seconds", ctypes.c_double), ("evaluations", ctypes.c_int64)]


@dataclass
class OracleSolution:
    status: int
    status_name: str
    iterations: int
    restarts: int
    objective: float
    dual_bound: float
    residuals: dict
    col_value: np.ndarray
    col_dual: np.ndarray
    row_dual: np.ndarray
    solve_seconds: float
    spectral_norm: float = float("nan")
    message: str = ""


class CQp(ctypes.Structure):
    _fields_ = [("lp", CLp), ("hessian_starts", _I), ("hessian_index", _I),
                ("hessian_values", _D)]


class CQpParams(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("iteration_limit", ctypes.c_int64),
                ("time_limit", ctypes.c_double), ("random_seed", ctypes.c_int64)]


class CQpResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("ceiling", ctypes.c_int32),
                ("iterations", ctypes.c_int64)] + [(k, ctypes.c_double) for k in (
                    "primal_residual", "dual_residual", "norm_a", "norm_q", "tau", "sigma",
                    "objective", "solve_seconds")]


@dataclass
class QpSolution:
    status: int
    status_name: str
    iterations: int
    objective: float
    col_value: np.ndarray
    col_dual: np.ndarray
    row_dual: np.ndarray
    solve_seconds: float
    primal_residual: float = float("nan")  # restatement only (the last check's)
    dual_residual: float = float("nan")
    norm_a: float = float("nan")
    norm_q: float = float("nan")
    tau: float = float("nan")
    sigma: float = float("nan")
    message: str = ""


def build(reference: bool = False) -> None:
    """Compile the restatement (always) and the reference library (when asked, from the
    reference tree or, on a machine without it, from its staged copy). A failure to build the
    reference from the staged copy is reported and left: the tests that need it skip, and the
    CPU baseline falls back to the restatement."""
    srcs = [os.path.join(HERE, f) for f in ("pdhg_oracle.c", "qp_oracle.c")]
    deps = srcs + [s[:-1] + "h" for s in srcs]
    if (not os.path.exists(ORACLE_LIB)
            or os.path.getmtime(ORACLE_LIB) < max(os.path.getmtime(d) for d in deps)):
        subprocess.run(["gcc", "-O2", "-fPIC", "-std=c11", "-ffp-contract=off", "-fopenmp",
                        "-shared", "-o", ORACLE_LIB] + srcs + ["-lm"], check=True)
    if not reference:
        return
    if os.path.isdir(os.path.join(REFERENCE_TREE, "src", "pdhg")):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "stage", f"REF={REFERENCE_TREE}"],
                       check=True)
    elif os.path.isdir(os.path.join(STAGE_TREE, "src", "pdhg")):
        proc = subprocess.run(["make", "-s", f"-j{os.cpu_count() or 8}", "-C", HERE, "ref",
                               f"REF={STAGE_TREE}"], stdout=subprocess.PIPE,
                              stderr=subprocess.STDOUT, text=True)
        if proc.returncode != 0:
            import sys

            sys.stderr.write("pyoracle: the reference library did not build from the staged "
                             "copy; its checks will skip\n" + proc.stdout[-2000:])


def reference_tree():
    """The reference checkout, else its staged copy, else None."""
    for tree in (REFERENCE_TREE, STAGE_TREE):
        if os.path.isdir(os.path.join(tree, "src", "pdhg")):
            return tree
    return None


def build_reference_gpu() -> str:
    """Compile the reference's own CUDA PDHG (`make -C oracle ref-gpu`) from the reference
    tree or its staged copy; returns the library's path. Raises when neither is present."""
    tree = reference_tree()
    if tree is None:
        raise RuntimeError("neither the reference tree nor its staged copy is present")
    subprocess.run(["make", "-s", "-j16", "-C", HERE, "ref-gpu", f"REF={tree}"], check=True,
                   stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return REF_GPU_LIB


def reference_gpu_solve(lp, tolerance, iteration_limit=-1, time_limit=None):
    """The reference's CUDA PDHG (src/gpu/pdhg_gpu.cu) on one LP, through
    ref/ref_gpu_capi.cpp. Returns a dict: status (the reference's SolveStatus value),
    iterations, objective, solve_seconds, primal / dual infeasibility and relative gap,
    algorithm ("pdhg-cuda" when the CUDA path ran to the end) and message."""
    lib = ctypes.CDLL(REF_GPU_LIB)
    f = lib.ref_gpu_solve_pdhg
    f.argtypes = [ctypes.POINTER(CLp), ctypes.c_double, ctypes.c_int64, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_int64), _D, _D, _D, ctypes.c_char_p, ctypes.c_int32,
                  ctypes.c_char_p, ctypes.c_int32]
    f.restype = ctypes.c_int32
    c, keep = Oracle._clp(lp)
    its = ctypes.c_int64()
    obj, sec = ctypes.c_double(), ctypes.c_double()
    res = np.zeros(3)
    alg = ctypes.create_string_buffer(64)
    msg = ctypes.create_string_buffer(512)
    status = f(ctypes.byref(c), tolerance, iteration_limit,
               1e308 if time_limit is None else time_limit, ctypes.byref(its),
               ctypes.byref(obj), ctypes.byref(sec), _ptr(res, ctypes.c_double), alg, 64, msg,
               512)
    del keep
    return {"status": int(status), "iterations": int(its.value), "objective": obj.value,
            "solve_seconds": sec.value, "primal_infeasibility": float(res[0]),
            "dual_infeasibility": float(res[1]), "relative_gap": float(res[2]),
            "algorithm": alg.value.decode(), "message": msg.value.decode()}


def reference_available() -> bool:
    return os.path.exists(REF_LIB)


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class Oracle:
    def __init__(self, reference: bool = False):
        path = REF_LIB if reference else ORACLE_LIB
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built")
        self.reference = reference
        self.lib = ctypes.CDLL(path)
        p = "ref_" if reference else "orc_"
        self._solve = getattr(self.lib, p + "solve_pdhg")
        if reference:
            self._solve.argtypes = [ctypes.POINTER(CLp), ctypes.POINTER(CParams),
                                    ctypes.POINTER(CResult), _D, _D, _D, ctypes.c_char_p,
                                    ctypes.c_int32]
        else:
            self._solve.argtypes = [ctypes.POINTER(CLp), ctypes.POINTER(CParams),
                                    ctypes.POINTER(CResult), _D, _D, _D]
        self._solve.restype = ctypes.c_int32
        self._scaling = getattr(self.lib, p + "build_scaling")
        self._scaling.argtypes = [ctypes.POINTER(CLp), _D, ctypes.c_int32] + [_D] * 10
        self._scaling.restype = None
        self._evaluate = getattr(self.lib, p + "evaluate")
        self._evaluate.argtypes = [ctypes.POINTER(CLp), _D, _D, _D, _D]
        self._evaluate.restype = CResiduals
        if reference:
            self._norm = self.lib.ref_spectral_norm
            self._norm.argtypes = [ctypes.POINTER(CLp), ctypes.c_int32, ctypes.c_uint32]
        else:
            self._norm = self.lib.orc_spectral_norm
            self._norm.argtypes = [ctypes.c_int32, ctypes.c_int32, _I, _I, _D, ctypes.c_int32,
                                   ctypes.c_uint32]
            self.lib.orc_multiply.argtypes = [ctypes.c_int32, ctypes.c_int32, _I, _I, _D, _D, _D]
            self.lib.orc_transpose_multiply.argtypes = [ctypes.c_int32, ctypes.c_int32, _I, _I,
                                                        _D, _D, _D]
            self.lib.orc_power_start.argtypes = [ctypes.c_uint32, ctypes.c_int32, _D]
        self._norm.restype = ctypes.c_double

    @staticmethod
    def _clp(lp):
        lp = lp.contiguous()
        c = CLp(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                _ptr(lp.row_index, ctypes.c_int32), _ptr(lp.values, ctypes.c_double),
                _ptr(lp.col_cost, ctypes.c_double), _ptr(lp.col_lower, ctypes.c_double),
                _ptr(lp.col_upper, ctypes.c_double), _ptr(lp.row_lower, ctypes.c_double),
                _ptr(lp.row_upper, ctypes.c_double), lp.sense, lp.objective_offset)
        return c, lp  # keep the arrays alive with the struct

    def solve(self, lp, tolerance=1e-8, iteration_limit=-1, time_limit=None, restart=True,
              stop_at_request=False, random_seed=0) -> OracleSolution:
        c, keep = self._clp(lp)
        params = CParams(tolerance, iteration_limit, 1e308 if time_limit is None else time_limit,
                         int(restart), int(stop_at_request), random_seed)
        res = CResult()
        x = np.zeros(lp.cols)
        d = np.zeros(lp.cols)
        y = np.zeros(lp.rows)
        args = [ctypes.byref(c), ctypes.byref(params), ctypes.byref(res), _ptr(x, ctypes.c_double),
                _ptr(d, ctypes.c_double), _ptr(y, ctypes.c_double)]
        message = ""
        if self.reference:
            buf = ctypes.create_string_buffer(4096)
            self._solve(*args, buf, 4096)
            message = buf.value.decode(errors="replace")
        else:
            self._solve(*args)
        del keep
        residuals = res.final_residuals.as_dict()
        if self.reference:
            # The reference's Solution carries no residuals: evaluate its reported point with
            # its own evaluate (row_dual = -sense * y, src/pdhg/pdhg.cpp:495-499).
            residuals = self.evaluate(lp, x, -lp.sense * y)[0]
        return OracleSolution(res.status, STATUS_NAMES.get(res.status, str(res.status)),
                              res.iterations, res.restarts, res.objective, res.dual_bound,
                              residuals, x, d, y, res.solve_seconds, res.spectral_norm, message)

    # ---- Convex QP (src/qp/qp_condat_vu.cpp; the restatement in qp_oracle.c) ----

    @staticmethod
    def _cqp(qp):
        qp = qp.contiguous()
        c, keep = Oracle._clp(qp.lp)
        cq = CQp(c, _ptr(qp.hessian_starts, ctypes.c_int32), _ptr(qp.hessian_index, ctypes.c_int32),
                 _ptr(qp.hessian_values, ctypes.c_double))
        return cq, (qp, keep)

    def solve_qp(self, qp, tolerance=1e-8, iteration_limit=-1, time_limit=None,
                 random_seed=0) -> QpSolution:
        """The reference's solve_convex_qp (reference=True: its own build, convexity gate
        included) or the restatement orc_solve_qp (which has no convexity gate)."""
        cq, keep = self._cqp(qp)
        params = CQpParams(tolerance, iteration_limit,
                           1e308 if time_limit is None else time_limit, random_seed)
        res = CQpResult()
        x = np.zeros(qp.cols)
        d = np.zeros(qp.cols)
        y = np.zeros(qp.rows)
        f = getattr(self.lib, ("ref_" if self.reference else "orc_") + "solve_qp")
        args = [ctypes.byref(cq), ctypes.byref(params), ctypes.byref(res),
                _ptr(x, ctypes.c_double), _ptr(d, ctypes.c_double), _ptr(y, ctypes.c_double)]
        message = ""
        if self.reference:
            f.argtypes = [ctypes.POINTER(CQp), ctypes.POINTER(CQpParams),
                          ctypes.POINTER(CQpResult), _D, _D, _D, ctypes.c_char_p, ctypes.c_int32]
            f.restype = ctypes.c_int32
            buf = ctypes.create_string_buffer(4096)
            f(*args, buf, 4096)
            message = buf.value.decode(errors="replace")
        else:
            f.argtypes = [ctypes.POINTER(CQp), ctypes.POINTER(CQpParams),
                          ctypes.POINTER(CQpResult), _D, _D, _D]
            f.restype = ctypes.c_int32
            f(*args)
        del keep
        out = QpSolution(res.status, STATUS_NAMES.get(res.status, str(res.status)),
                         res.iterations, res.objective, x, d, y, res.solve_seconds,
                         message=message)
        if not self.reference:
            for k in ("primal_residual", "dual_residual", "norm_a", "norm_q", "tau", "sigma"):
                setattr(out, k, getattr(res, k))
        return out

    def qp_norms(self, qp, seed=0):
        """(||A||, ||Q||) by the QP engine's two power iterations (restatement only)."""
        cq, keep = self._cqp(qp)
        q = keep[0]
        self.lib.orc_qp_spectral_norm.argtypes = [ctypes.c_int32, ctypes.c_int32, _I, _I, _D,
                                                  ctypes.c_uint32]
        self.lib.orc_qp_spectral_norm.restype = ctypes.c_double
        self.lib.orc_qp_hessian_norm.argtypes = [ctypes.POINTER(CQp), ctypes.c_uint32]
        self.lib.orc_qp_hessian_norm.restype = ctypes.c_double
        a = self.lib.orc_qp_spectral_norm(q.rows, q.cols, cq.lp.col_starts, cq.lp.row_index,
                                          cq.lp.values, seed)
        return a, self.lib.orc_qp_hessian_norm(ctypes.byref(cq), seed)

    def check_convexity(self, qp):
        """(verdict, detail) of the reference's check_convexity (src/qp/convexity.cpp:177):
        0 convex, 1 indefinite, 2 unverified. Reference only."""
        cq, keep = self._cqp(qp)
        f = self.lib.ref_check_convexity
        f.argtypes = [ctypes.POINTER(CQp), ctypes.c_char_p, ctypes.c_int32]
        f.restype = ctypes.c_int32
        buf = ctypes.create_string_buffer(1024)
        verdict = f(ctypes.byref(cq), buf, 1024)
        return verdict, buf.value.decode(errors="replace")

    def build_scaling(self, lp, ruiz_iterations=10):
        c, keep = self._clp(lp)
        m, n = lp.rows, lp.cols
        out = dict(values=np.zeros(lp.nnz), row=np.zeros(m), col=np.zeros(n), cost=np.zeros(n),
                   col_lower=np.zeros(n), col_upper=np.zeros(n), row_lower=np.zeros(m),
                   row_upper=np.zeros(m))
        mn, mx = ctypes.c_double(), ctypes.c_double()
        cost = np.ascontiguousarray(lp.sense * np.asarray(lp.col_cost, dtype=np.float64))
        self._scaling(ctypes.byref(c), _ptr(cost, ctypes.c_double), ruiz_iterations,
                      *[_ptr(out[k], ctypes.c_double) for k in (
                          "values", "row", "col", "cost", "col_lower", "col_upper", "row_lower",
                          "row_upper")], ctypes.byref(mn), ctypes.byref(mx))
        del keep
        out["min_abs"], out["max_abs"] = mn.value, mx.value
        return out

    def spectral_norm(self, lp, iterations=30, seed=1):
        c, keep = self._clp(lp)
        if self.reference:
            return self._norm(ctypes.byref(c), iterations, seed)
        return self._norm(lp.rows, lp.cols, c.col_starts, c.row_index, c.values, iterations, seed)

    def evaluate(self, lp, x, y):
        c, keep = self._clp(lp)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        act = np.zeros(lp.rows)
        red = np.zeros(lp.cols)
        r = self._evaluate(ctypes.byref(c), _ptr(x, ctypes.c_double), _ptr(y, ctypes.c_double),
                           _ptr(act, ctypes.c_double), _ptr(red, ctypes.c_double))
        return r.as_dict(), act, red

    def multiply(self, lp, x):
        """y = A x (SparseMatrix::multiply)."""
        lp = lp.contiguous()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(lp.rows)
        if self.reference:
            c, keep = self._clp(lp)
            self.lib.ref_multiply.argtypes = [ctypes.POINTER(CLp), _D, _D]
            self.lib.ref_multiply.restype = None
            self.lib.ref_multiply(ctypes.byref(c), _ptr(x, ctypes.c_double),
                                  _ptr(y, ctypes.c_double))
            return y
        self.lib.orc_multiply(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                              _ptr(lp.row_index, ctypes.c_int32), _ptr(lp.values, ctypes.c_double),
                              _ptr(x, ctypes.c_double), _ptr(y, ctypes.c_double))
        return y

    def transpose_multiply(self, lp, y):
        """x = A^T y (SparseMatrix::transpose_multiply)."""
        lp = lp.contiguous()
        y = np.ascontiguousarray(y, dtype=np.float64)
        x = np.zeros(lp.cols)
        if self.reference:
            c, keep = self._clp(lp)
            self.lib.ref_transpose_multiply.argtypes = [ctypes.POINTER(CLp), _D, _D]
            self.lib.ref_transpose_multiply.restype = None
            self.lib.ref_transpose_multiply(ctypes.byref(c), _ptr(y, ctypes.c_double),
                                            _ptr(x, ctypes.c_double))
            return x
        self.lib.orc_transpose_multiply(lp.rows, lp.cols, _ptr(lp.col_starts, ctypes.c_int32),
                                        _ptr(lp.row_index, ctypes.c_int32),
                                        _ptr(lp.values, ctypes.c_double), _ptr(y, ctypes.c_double),
                                        _ptr(x, ctypes.c_double))
        return x

    # Restatement-only helper.

    def power_start(self, seed, count):
        out = np.zeros(count)
        self.lib.orc_power_start(seed, count, _ptr(out, ctypes.c_double))
        return out

    # Reference-only helpers: Models built by the reference's own code.
    def _model_from_handle(self, handle, name):
        from sankhya_gb300.model import LP

        lib = self.lib
        rows, cols = ctypes.c_int32(), ctypes.c_int32()
        nnz, optimum = ctypes.c_int64(), ctypes.c_int64()
        sense, offset = ctypes.c_double(), ctypes.c_double()
        lib.ref_model_shape(handle, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz),
                            ctypes.byref(sense), ctypes.byref(offset), ctypes.byref(optimum))
        m, n, z = rows.value, cols.value, nnz.value
        starts = np.zeros(n + 1, np.int32)
        index = np.zeros(z, np.int32)
        arrays = [np.zeros(k) for k in (z, n, n, n, m, m)]
        lib.ref_model_arrays(handle, _ptr(starts, ctypes.c_int32), _ptr(index, ctypes.c_int32),
                             *[_ptr(a, ctypes.c_double) for a in arrays])
        lib.ref_model_free(handle)
        values, cost, lower, upper, row_lower, row_upper = arrays
        lp = LP(m, n, starts, index, values, cost, lower, upper, row_lower, row_upper,
                sense=sense.value, objective_offset=offset.value, name=name)
        return lp, optimum.value

    def _model_api(self):
        if not self.reference:
            raise RuntimeError("only the reference library reads and generates Models")
        lib = self.lib
        lib.ref_model_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
        lib.ref_model_read.restype = ctypes.c_void_p
        lib.ref_model_kkt_lp.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32]
        lib.ref_model_kkt_lp.restype = ctypes.c_void_p
        lib.ref_model_shape.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 6
        lib.ref_model_shape.restype = None
        lib.ref_model_arrays.argtypes = [ctypes.c_void_p, _I, _I] + [_D] * 6
        lib.ref_model_arrays.restype = None
        lib.ref_model_free.argtypes = [ctypes.c_void_p]
        lib.ref_model_free.restype = None
        return lib

    def read_model(self, path):
        """The LP in an MPS or LP file, as the reference's reader builds it
        (sankhya::io::read_model, src/io/lp_reader.cpp:650)."""
        lib = self._model_api()
        err = ctypes.create_string_buffer(1024)
        handle = lib.ref_model_read(os.fsencode(path), err, 1024)
        if not handle:
            raise ValueError(f"{path}: {err.value.decode(errors='replace')}")
        return self._model_from_handle(handle, os.path.basename(path))[0]

    def read_qp(self, path):
        """The QP in an MPS file with a QUADOBJ section, as the reference's reader builds it:
        the LP part and Model::hessian's stored triangle."""
        from sankhya_gb300.model import QP

        lib = self._model_api()
        lib.ref_model_hessian_nonzeros.argtypes = [ctypes.c_void_p]
        lib.ref_model_hessian_nonzeros.restype = ctypes.c_int64
        lib.ref_model_hessian.argtypes = [ctypes.c_void_p, _I, _I, _D]
        lib.ref_model_hessian.restype = None
        err = ctypes.create_string_buffer(1024)
        handle = lib.ref_model_read(os.fsencode(path), err, 1024)
        if not handle:
            raise ValueError(f"{path}: {err.value.decode(errors='replace')}")
        rows, cols = ctypes.c_int32(), ctypes.c_int32()
        nnz, optimum = ctypes.c_int64(), ctypes.c_int64()
        sense, offset = ctypes.c_double(), ctypes.c_double()
        lib.ref_model_shape(handle, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz),
                            ctypes.byref(sense), ctypes.byref(offset), ctypes.byref(optimum))
        hz = lib.ref_model_hessian_nonzeros(handle)
        hs = np.zeros(cols.value + 1, np.int32)
        hi = np.zeros(hz, np.int32)
        hv = np.zeros(hz)
        lib.ref_model_hessian(handle, _ptr(hs, ctypes.c_int32), _ptr(hi, ctypes.c_int32),
                              _ptr(hv, ctypes.c_double))
        lp = self._model_from_handle(handle, os.path.basename(path))[0]
        return QP(lp, hs, hi, hv, os.path.basename(path))

    def kkt_lp(self, seed, trial, max_rows=8, max_cols=8):
        """(LP, exact optimal objective): the trial-th instance of the reference's generator
        of LPs with a known optimum (sankhya::oracle::kkt_lp, tests/oracles/lp_generator.cpp:122)
        drawn from one mt19937_64(seed)."""
        lib = self._model_api()
        handle = lib.ref_model_kkt_lp(seed, trial, max_rows, max_cols)
        return self._model_from_handle(handle, f"kkt_lp_{seed}_{trial}")

"""The LP as SANKHYA's Model holds it, in numpy arrays.

Mirrors the fields of ``sankhya::Model`` that an LP engine reads
(include/sankhya/model.hpp:123-170 in the reference): a CSC matrix with int32 column starts,
ascending int32 row indices and FP64 values; two-sided rows ``rl <= A x <= ru``; column
bounds ``l <= x <= u``; the objective sense and constant offset. ``+-inf`` (or any magnitude
at or above 1e30) means "no bound", as ``is_finite_bound`` (include/sankhya/types.hpp:88-96)
defines it.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np


@dataclass
class LP:
    rows: int
    cols: int
    col_starts: np.ndarray  # int32, cols + 1
    row_index: np.ndarray  # int32, nnz
    values: np.ndarray  # float64, nnz
    col_cost: np.ndarray
    col_lower: np.ndarray
    col_upper: np.ndarray
    row_lower: np.ndarray
    row_upper: np.ndarray
    sense: float = 1.0  # +1 minimise, -1 maximise (Model::sense_multiplier)
    objective_offset: float = 0.0
    # Planted optimum, when the generator knows it (minimise-space objective value).
    x0: Optional[np.ndarray] = None
    lam: Optional[np.ndarray] = None
    fstar: Optional[float] = None
    name: str = field(default="lp")

    @property
    def nnz(self) -> int:
        return int(self.col_starts[-1])

    def validate(self) -> str:
        """Shape checks in the spirit of Model::validate (src/core/model.cpp:127-240)."""
        if len(self.col_starts) != self.cols + 1:
            return "col_starts length != num_cols + 1"
        for name in ("col_cost", "col_lower", "col_upper"):
            if len(getattr(self, name)) != self.cols:
                return f"{name} length != num_cols"
        for name in ("row_lower", "row_upper"):
            if len(getattr(self, name)) != self.rows:
                return f"{name} length != num_rows"
        if len(self.row_index) != self.nnz or len(self.values) != self.nnz:
            return "row_index / values length != nnz"
        return ""

    def contiguous(self) -> "LP":
        """The same LP with every array C-contiguous in the dtype the C ABI expects."""
        def f64(a):
            return np.ascontiguousarray(a, dtype=np.float64)

        def i32(a):
            return np.ascontiguousarray(a, dtype=np.int32)

        return LP(self.rows, self.cols, i32(self.col_starts), i32(self.row_index),
                  f64(self.values), f64(self.col_cost), f64(self.col_lower), f64(self.col_upper),
                  f64(self.row_lower), f64(self.row_upper), float(self.sense),
                  float(self.objective_offset), self.x0, self.lam, self.fstar, self.name)

    def to_dense(self) -> np.ndarray:
        a = np.zeros((self.rows, self.cols))
        for j in range(self.cols):
            for k in range(self.col_starts[j], self.col_starts[j + 1]):
                a[self.row_index[k], j] += self.values[k]
        return a


def from_dense(a, row_lower, row_upper, cost, col_lower=None, col_upper=None, sense=1.0,
               offset=0.0, name="dense") -> LP:
    """Build an LP from a dense matrix (zeros dropped), as the reference tests' make_lp does
    (tests/unit/test_pdhg.cpp:66-91): columns default to 0 <= x < inf."""
    a = np.asarray(a, dtype=np.float64)
    m, n = a.shape
    starts = [0]
    rows, vals = [], []
    for j in range(n):
        for i in range(m):
            if a[i, j] != 0.0:
                rows.append(i)
                vals.append(a[i, j])
        starts.append(len(rows))
    lo = np.zeros(n) if col_lower is None else np.asarray(col_lower, dtype=np.float64)
    hi = np.full(n, np.inf) if col_upper is None else np.asarray(col_upper, dtype=np.float64)
    return LP(m, n, np.array(starts, dtype=np.int32), np.array(rows, dtype=np.int32),
              np.array(vals, dtype=np.float64), np.asarray(cost, dtype=np.float64), lo, hi,
              np.asarray(row_lower, dtype=np.float64), np.asarray(row_upper, dtype=np.float64),
              float(sense), float(offset), name=name)

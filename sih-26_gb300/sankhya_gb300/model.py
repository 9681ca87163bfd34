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


@dataclass
class QP:
    """A convex QP as ``sankhya::Model`` holds it: the LP part and ``Model::hessian``, the
    stored lower triangle of the symmetric Q as an n x n CSC (int32 starts and indices, FP64
    values). The objective is ``offset + c'x + 0.5 x'Qx``: a stored off-diagonal entry (i, j)
    stands for both Q_ij and Q_ji (include/sankhya/model.hpp, src/core/model.cpp:101-125)."""
    lp: LP
    hessian_starts: np.ndarray  # int32, cols + 1
    hessian_index: np.ndarray  # int32
    hessian_values: np.ndarray  # float64
    name: str = field(default="qp")

    @property
    def rows(self) -> int:
        return self.lp.rows

    @property
    def cols(self) -> int:
        return self.lp.cols

    @property
    def hessian_nnz(self) -> int:
        return int(self.hessian_starts[-1])

    def contiguous(self) -> "QP":
        return QP(self.lp.contiguous(), np.ascontiguousarray(self.hessian_starts, dtype=np.int32),
                  np.ascontiguousarray(self.hessian_index, dtype=np.int32),
                  np.ascontiguousarray(self.hessian_values, dtype=np.float64), self.name)

    def hessian_dense(self) -> np.ndarray:
        """The full symmetric Q."""
        n = self.cols
        q = np.zeros((n, n))
        for j in range(n):
            for k in range(self.hessian_starts[j], self.hessian_starts[j + 1]):
                i = self.hessian_index[k]
                q[i, j] += self.hessian_values[k]
                if i != j:
                    q[j, i] += self.hessian_values[k]
        return q

    def objective(self, x) -> float:
        """Model::evaluate_objective (src/core/model.cpp:101-125), vectorised."""
        x = np.asarray(x, dtype=np.float64)
        lin = self.lp.objective_offset + float(np.dot(self.lp.col_cost, x))
        cols = np.repeat(np.arange(self.cols), np.diff(self.hessian_starts))
        rows = np.asarray(self.hessian_index)
        v = np.asarray(self.hessian_values)
        w = np.where(rows == cols, 0.5, 1.0)
        return lin + float(np.sum(w * v * x[rows] * x[cols]))


def hessian_from_triples(n, triples):
    """CSC of the stored triangle from (row, col, value) triples, as the reference tests'
    make_qp builds Model::hessian (tests/unit/test_qp.cpp:34-68): add_entry then finalize, so
    each column's rows come out ascending."""
    by_col = [[] for _ in range(n)]
    for i, j, v in triples:
        by_col[j].append((i, v))
    starts, index, values = [0], [], []
    for j in range(n):
        for i, v in sorted(by_col[j]):
            index.append(i)
            values.append(v)
        starts.append(len(index))
    return (np.array(starts, dtype=np.int32), np.array(index, dtype=np.int32),
            np.array(values, dtype=np.float64))


def qp_from_dense(cost, col_lower, col_upper, hessian_lower, rows=(), row_lower=(),
                  row_upper=(), sense=1.0, offset=0.0, name="qp") -> QP:
    """make_qp of tests/unit/test_qp.cpp:34-68: cost, column bounds, the Hessian's stored
    lower triangle as (row, col, value) triples, and dense rows with their bounds."""
    n = len(cost)
    a = np.zeros((len(rows), n)) if len(rows) == 0 else np.asarray(rows, dtype=np.float64)
    lp = from_dense(a.reshape(len(rows), n), row_lower, row_upper, cost, col_lower, col_upper,
                    sense=sense, offset=offset, name=name)
    hs, hi, hv = hessian_from_triples(n, hessian_lower)
    return QP(lp, hs, hi, hv, name)


def random_qp(seed, rows, cols, per_column=4, hessian_band=2, equality_share=0.3,
              maximise=False, name=None) -> QP:
    """A seeded convex QP with a strictly feasible point.

    A has `per_column` N(0, 1) entries per column at distinct random rows; Q = D + the band
    of `hessian_band` sub-diagonals with N(0, 0.3) entries, its diagonal D raised to make Q
    diagonally dominant (so positive definite); columns in [-5, 5], some free or one-sided;
    rows around A x0 for a random x0 in the box: a share of them equalities, the rest one- or
    two-sided with slack. maximise=True negates c and Q (a concave maximisation: the same
    minimiser)."""
    rng = np.random.default_rng(seed)
    m, n = rows, cols
    starts, index, values = [0], [], []
    for j in range(n):
        k = min(per_column, m)
        r = np.sort(rng.choice(m, size=k, replace=False)) if m > 0 else np.array([], int)
        index.extend(r.tolist())
        values.extend(rng.normal(size=len(r)).tolist())
        starts.append(len(index))
    starts = np.array(starts, dtype=np.int32)
    index = np.array(index, dtype=np.int32)
    values = np.array(values, dtype=np.float64)
    lower = np.full(n, -5.0)
    upper = np.full(n, 5.0)
    kind = rng.integers(0, 4, size=n)
    lower[kind == 1] = -np.inf
    upper[kind == 2] = np.inf
    lower[kind == 3], upper[kind == 3] = -np.inf, np.inf
    x0 = rng.uniform(-2.0, 2.0, size=n)
    ax = np.zeros(m)
    for j in range(n):
        ax[index[starts[j]:starts[j + 1]]] += values[starts[j]:starts[j + 1]] * x0[j]
    row_lower = ax - rng.uniform(0.1, 1.0, size=m)
    row_upper = ax + rng.uniform(0.1, 1.0, size=m)
    eq = rng.random(m) < equality_share
    row_lower[eq] = row_upper[eq] = ax[eq]
    one = (~eq) & (rng.random(m) < 0.5)
    row_upper[one & (rng.random(m) < 0.5)] = np.inf
    row_lower[one & ~np.isinf(row_upper)] = -np.inf
    cost = rng.normal(size=n)
    # Hessian: band entries below the diagonal, then a dominant diagonal.
    triples = []
    off = np.zeros(n)
    for b in range(1, hessian_band + 1):
        for j in range(n - b):
            v = 0.3 * rng.normal()
            triples.append((j + b, j, v))
            off[j] += abs(v)
            off[j + b] += abs(v)
    for j in range(n):
        triples.append((j, j, off[j] + rng.uniform(0.2, 2.0)))
    hs, hi, hv = hessian_from_triples(n, triples)
    sense = 1.0
    if maximise:
        cost, hv, sense = -cost, -hv, -1.0
    lp = LP(m, n, starts, index, values, cost, lower, upper, row_lower, row_upper,
            sense=sense, name=name or f"random_qp_{seed}")
    return QP(lp, hs, hi, hv, lp.name)


def banded_hessian(n, band=2, seed=0, scale=0.3):
    """The stored lower triangle (CSC) of a positive definite banded Q of order n: entries
    (j + b, j) for b = 1..band drawn from N(0, scale^2), and a diagonal raised above the sum of
    each row's off-diagonal magnitudes by U(0.2, 2). Vectorised, for the QP workloads."""
    rng = np.random.default_rng(seed)
    j = np.arange(n)
    vals = np.zeros((n, band + 1))
    rowsum = np.zeros(n)
    for b in range(1, band + 1):
        v = scale * rng.normal(size=max(n - b, 0))
        vals[: n - b, b] = v
        rowsum[: n - b] += np.abs(v)
        rowsum[b:] += np.abs(v)
    vals[:, 0] = rowsum + rng.uniform(0.2, 2.0, size=n)
    rows = j[:, None] + np.arange(band + 1)[None, :]
    valid = rows < n
    counts = valid.sum(axis=1)
    starts = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=starts[1:])
    return (starts.astype(np.int32), rows[valid].astype(np.int32),
            vals[valid].astype(np.float64))

"""The synthetic generators plant a KKT point: the oracle's evaluate (the reference's
residual formula) at (x0, -lambda) must be ~0 on every residual."""
import numpy as np
import pytest

from sankhya_gb300 import lpgen


@pytest.mark.parametrize("make", [
    lambda: lpgen.planted_uniform(300, 700, 5, seed=1),
    lambda: lpgen.planted_blocks(5, 40, 80, 9, seed=2),
    lambda: lpgen.planted_general(80, 120, 3, seed=3),
    lambda: lpgen.planted_zipf(300, 600, 6000, max_len=400, seed=4),
])
def test_planted_point_is_optimal(oracle, make):
    lp = make()
    # The engine's y is the NEGATIVE of the row multiplier (src/pdhg/pdhg.cpp:34-37).
    r, act, red = oracle.evaluate(lp, lp.x0, -lp.lam)
    assert r["absolute_primal"] < 1e-9
    assert r["absolute_dual"] < 1e-9
    assert r["gap_as_verified"] < 1e-12
    assert r["complementarity"] < 1e-9
    assert abs(r["primal_objective"] - lp.fstar) <= 1e-12 * max(1, abs(lp.fstar))


def test_shapes():
    lp = lpgen.planted_uniform(50, 120, 5, seed=4)
    assert lp.nnz == 600 and lp.validate() == ""
    assert np.all(np.diff(lp.col_starts) == 5)
    for j in range(lp.cols):
        rows = lp.row_index[lp.col_starts[j]:lp.col_starts[j + 1]]
        assert np.all(np.diff(rows) > 0)
    b = lpgen.planted_blocks(3, 10, 20, 4, seed=5)
    assert b.rows == 30 and b.cols == 60 and b.nnz == 60 * 4 + 40
    # Linking entries are +-1 and fall in the next block.
    for j in range(40):
        k1 = b.col_starts[j + 1] - 1
        assert abs(b.values[k1]) == 1.0 and b.row_index[k1] // 10 == j // 20 + 1


def test_determinism():
    a = lpgen.planted_uniform(100, 200, 5, seed=9)
    b = lpgen.planted_uniform(100, 200, 5, seed=9)
    assert np.array_equal(a.values, b.values) and np.array_equal(a.col_cost, b.col_cost)
    c = lpgen.planted_uniform(100, 200, 5, seed=10)
    assert not np.array_equal(a.values, c.values)


def test_zipf_shape():
    lp = lpgen.planted_zipf(2000, 4000, 40000, max_len=1000, seed=3)
    assert lp.validate() == ""
    assert abs(lp.nnz - 40000) < 0.1 * 40000
    lens = np.bincount(lp.row_index, minlength=lp.rows)
    assert lens.min() >= 2 and lens.max() <= 1000
    # Heavy tail: the median row is short, the longest rows are far longer.
    assert np.median(lens) <= 4 and lens.max() >= 50 * np.median(lens)
    mag = np.abs(lp.values)
    assert mag.min() >= 1e-3 * (1 - 1e-12) and mag.max() <= 1e3 * (1 + 1e-12)
    assert (lp.values < 0).mean() > 0.4 and (lp.values > 0).mean() > 0.4
    for j in range(0, lp.cols, 97):
        rows = lp.row_index[lp.col_starts[j]:lp.col_starts[j + 1]]
        assert np.all(np.diff(rows) > 0)
    again = lpgen.planted_zipf(2000, 4000, 40000, max_len=1000, seed=3)
    assert np.array_equal(lp.values, again.values) and np.array_equal(lp.row_index,
                                                                      again.row_index)

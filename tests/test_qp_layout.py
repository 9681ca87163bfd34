"""The convex-QP engine's host layouts (sih-26_gb300/csrc/qp_layout.hpp, the functions
QpEngine::load and QpEngine::layout call), checked on the CPU through
tests/host/qp_layout_export.cpp against an independent numpy build:

* A by rows equals the CSR of the CSC, columns ascending in each row;
* sense Q by rows holds both triangles of the stored one (an off-diagonal entry twice, the
  diagonal once), columns ascending, whatever triangle the entries were stored in;
* the lengths per column (Q row + A column) and per row;
* the cost times the sense, absent bounds (infinite or of magnitude >= 1e30) as infinities;
* the chunk table: exactly the items longer than 64 lanes' worth, cut into consecutive chunks
  of at most 2,048 entries that cover the item, with consistent first / count / slot;
* the lanes rule.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from sankhya_gb300.model import QP, hessian_from_triples, random_qp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("qp_layout") / "libqplayout.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "sih-26_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host", "qp_layout_export.cpp"), "-o", out],
                   check=True)
    return ctypes.CDLL(out)


def _layout(lib, qp):
    from sankhya_gb300.capi import CLp, CQpProblem

    qp = qp.contiguous()
    lp = qp.lp

    def p(a, t=ctypes.c_double):
        return a.ctypes.data_as(ctypes.POINTER(t))

    c = CLp(lp.rows, lp.cols, p(lp.col_starts, ctypes.c_int32), p(lp.row_index, ctypes.c_int32),
            p(lp.values), p(lp.col_cost), p(lp.col_lower), p(lp.col_upper), p(lp.row_lower),
            p(lp.row_upper), lp.sense, lp.objective_offset)
    prob = CQpProblem(c, p(qp.hessian_starts, ctypes.c_int32),
                      p(qp.hessian_index, ctypes.c_int32), p(qp.hessian_values))
    rz, qz = ctypes.c_longlong(), ctypes.c_longlong()
    lib.qp_layout_sizes(ctypes.byref(prob), ctypes.byref(rz), ctypes.byref(qz))
    m, n = lp.rows, lp.cols
    out = {"row_starts": np.zeros(m + 1, np.int32), "row_cols": np.zeros(rz.value, np.int32),
           "row_values": np.zeros(rz.value), "q_starts": np.zeros(n + 1, np.int32),
           "q_cols": np.zeros(qz.value, np.int32), "q_values": np.zeros(qz.value),
           "col_len": np.zeros(n, np.int32), "row_len": np.zeros(m, np.int32),
           "cost": np.zeros(n), "col_lower": np.zeros(n), "col_upper": np.zeros(n),
           "row_lower": np.zeros(m), "row_upper": np.zeros(m)}
    args = [p(v, ctypes.c_int32) if v.dtype == np.int32 else p(v) for v in out.values()]
    lib.qp_layout_fill(ctypes.byref(prob), *args)
    return qp, out


def _csr(starts, cols, values, rows, ncols):
    dense = np.zeros((rows, ncols))
    for r in range(rows):
        seg = slice(starts[r], starts[r + 1])
        assert np.all(np.diff(cols[seg]) >= 0), "columns ascending in each row"
        np.add.at(dense[r], cols[seg], values[seg])
    return dense


@pytest.mark.parametrize("make", [
    lambda: random_qp(71, 40, 70),
    lambda: random_qp(72, 30, 50, maximise=True),
    lambda: random_qp(73, 0, 20),
], ids=["min", "max", "no_rows"])
def test_layout_matches_numpy(lib, make):
    qp, out = _layout(lib, make())
    lp = qp.lp
    m, n = lp.rows, lp.cols
    a = lp.to_dense()
    assert np.array_equal(_csr(out["row_starts"], out["row_cols"], out["row_values"], m, n), a)
    q = qp.hessian_dense()
    assert np.array_equal(_csr(out["q_starts"], out["q_cols"], out["q_values"], n, n),
                          lp.sense * q)
    stored = np.diff(qp.hessian_starts)
    diag = sum(1 for j in range(n) for k in range(qp.hessian_starts[j], qp.hessian_starts[j + 1])
               if qp.hessian_index[k] == j)
    assert out["q_starts"][-1] == 2 * int(stored.sum()) - diag
    assert np.array_equal(out["col_len"], np.diff(out["q_starts"]) + np.diff(lp.col_starts))
    assert np.array_equal(out["row_len"], np.diff(out["row_starts"]))
    assert np.array_equal(out["cost"], lp.sense * lp.col_cost)

    def norm(v, side):
        v = np.asarray(v, dtype=np.float64)
        absent = np.isinf(v) | (np.abs(v) >= 1e30)
        return np.where(absent, side * np.inf, v)

    assert np.array_equal(out["col_lower"], norm(lp.col_lower, -1))
    assert np.array_equal(out["col_upper"], norm(lp.col_upper, 1))
    assert np.array_equal(out["row_lower"], norm(lp.row_lower, -1))
    assert np.array_equal(out["row_upper"], norm(lp.row_upper, 1))


def test_layout_upper_triangle_and_absent_bounds(lib):
    """Entries stored above the diagonal are expanded like their mirrors and sorted into place;
    bounds of magnitude 1e30 are absent on either side."""
    base = random_qp(74, 12, 9)
    lp = base.lp
    lp.col_lower[0], lp.col_upper[1] = 1e30, -1e30
    lp.row_lower[0], lp.row_upper[1] = -1e31, np.inf
    triples = [(j, j, 3.0 + j) for j in range(9)] + [(0, 5, 0.5), (2, 7, -0.25), (8, 1, 0.125)]
    hs, hi, hv = hessian_from_triples(9, triples)
    qp, out = _layout(lib, QP(lp, hs, hi, hv))
    q = np.diag([3.0 + j for j in range(9)])
    for i, j, v in triples[9:]:
        q[i, j] += v
        q[j, i] += v
    assert np.array_equal(_csr(out["q_starts"], out["q_cols"], out["q_values"], 9, 9), q)
    assert out["col_lower"][0] == -np.inf and out["col_upper"][1] == np.inf
    assert out["row_lower"][0] == -np.inf and out["row_upper"][1] == np.inf


@pytest.mark.parametrize("lanes", [1, 2, 8, 32])
def test_chunk_table(lib, lanes):
    rng = np.random.default_rng(lanes)
    lengths = np.concatenate([rng.integers(0, 80, 500), [64 * lanes, 64 * lanes + 1, 2048,
                                                         2049, 4096, 10000, 123457]])
    rng.shuffle(lengths)
    lengths = lengths.astype(np.int32)
    cap = 4096
    out = np.zeros(6 * cap, np.int32)
    nlong = ctypes.c_int32()
    count = lib.qp_layout_chunks(lengths.ctypes.data_as(_I), len(lengths), lanes,
                                 out.ctypes.data_as(_I), cap, ctypes.byref(nlong))
    assert count >= 0
    chunks = out[:6 * count].reshape(count, 6)
    long_items = [i for i, l in enumerate(lengths) if l > 64 * lanes]
    assert nlong.value == len(long_items)
    at = 0
    for slot, item in enumerate(long_items):
        l = int(lengths[item])
        want = (l + 2047) // 2048
        rows = chunks[at:at + want]
        assert np.all(rows[:, 0] == item) and np.all(rows[:, 3] == at)
        assert np.all(rows[:, 4] == want) and np.all(rows[:, 5] == slot)
        assert rows[0, 1] == 0 and rows[-1, 2] == l
        assert np.all(rows[1:, 1] == rows[:-1, 2])
        assert np.all(rows[:, 2] - rows[:, 1] <= 2048) and np.all(rows[:, 2] > rows[:, 1])
        at += want
    assert at == count


def test_lanes_rule(lib):
    lib.qp_layout_lanes.restype = ctypes.c_int
    lib.qp_layout_lanes.argtypes = [ctypes.c_double]
    got = [lib.qp_layout_lanes(v) for v in (1.0, 15.0, 20.0, 32.0, 33.0, 64.0, 65.0, 1e4)]
    assert got == [1, 1, 1, 1, 2, 2, 4, 32]

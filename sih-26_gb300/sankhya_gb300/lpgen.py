"""Seeded planted-optimum LP generators (ctypes over lpgen/lpgen.c).

The shapes follow the synthetic workloads this engine is measured on:

* ``planted_uniform(m, n, k, seed)`` -- m x n, exactly k distinct uniform rows per column,
  N(0,1) values, equality rows, 0 <= x <= 10 (the 2,000 x 5,000 parity case, the batched
  and the differentiation cases).
* ``planted_blocks(blocks, R, C, k, seed)`` -- block-angular multi-period structure with one
  +-1 inventory link per column into the next period (64 x 15,625 x 31,250 with k = 9 is the
  1,000,000 x 2,000,000 headline case).
* ``planted_zipf(m, n, target_nnz, ...)`` -- Zipf-distributed row lengths, uniform columns,
  badly scaled values (500,000 x 1,000,000 with about 3e7 nonzeros is the load-balance
  stress case).
* ``planted_general(m, n, k, seed)`` -- every row and column kind, for coverage.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _paths
from .model import LP

_lib = None


class _CLp(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("nnz", ctypes.c_int64),
        ("col_starts", ctypes.c_void_p), ("row_index", ctypes.c_void_p),
        ("values", ctypes.c_void_p), ("col_cost", ctypes.c_void_p),
        ("col_lower", ctypes.c_void_p), ("col_upper", ctypes.c_void_p),
        ("row_lower", ctypes.c_void_p), ("row_upper", ctypes.c_void_p),
        ("x0", ctypes.c_void_p), ("lam", ctypes.c_void_p), ("fstar", ctypes.c_double),
    ]


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_paths.LPGEN_LIB):
            # The generators are plain C and compile in a second, so a fresh checkout (or a
            # test collection that runs before build()) builds them on first use.
            from . import build

            build.build_lpgen()
        lib = ctypes.CDLL(_paths.LPGEN_LIB)
        for name in ("lpgen_planted_uniform", "lpgen_planted_general",
                     "lpgen_planted_nondegenerate"):
            getattr(lib, name + "_nnz").argtypes = [ctypes.c_int32] * 3
            getattr(lib, name + "_nnz").restype = ctypes.c_int64
            getattr(lib, name).restype = ctypes.c_int32
        lib.lpgen_planted_uniform.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_uint64,
                                                                     ctypes.POINTER(_CLp)]
        lib.lpgen_planted_general.argtypes = [ctypes.c_int32] * 4 + [ctypes.c_uint64,
                                                                     ctypes.POINTER(_CLp)]
        lib.lpgen_planted_nondegenerate.argtypes = [ctypes.c_int32] * 3 + [
            ctypes.c_uint64, ctypes.POINTER(_CLp)]
        lib.lpgen_planted_blocks.argtypes = [ctypes.c_int32] * 4 + [ctypes.c_uint64,
                                                                    ctypes.POINTER(_CLp)]
        lib.lpgen_planted_blocks.restype = ctypes.c_int32
        lib.lpgen_planted_blocks_nnz.argtypes = [ctypes.c_int32] * 4
        lib.lpgen_planted_blocks_nnz.restype = ctypes.c_int64
        lib.lpgen_planted_zipf_nnz.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
                                               ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_uint64]
        lib.lpgen_planted_zipf_nnz.restype = ctypes.c_int64
        lib.lpgen_planted_zipf.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
                                           ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_uint64, ctypes.POINTER(_CLp)]
        lib.lpgen_planted_zipf.restype = ctypes.c_int32
        _lib = lib
    return _lib


def _alloc(m, n, nnz):
    arrays = dict(
        col_starts=np.zeros(n + 1, np.int32), row_index=np.zeros(nnz, np.int32),
        values=np.zeros(nnz), col_cost=np.zeros(n), col_lower=np.zeros(n),
        col_upper=np.zeros(n), row_lower=np.zeros(m), row_upper=np.zeros(m), x0=np.zeros(n),
        lam=np.zeros(m))
    c = _CLp()
    for key, arr in arrays.items():
        setattr(c, key, arr.ctypes.data)
    return arrays, c


def _finish(arrays, c, name, sense=1.0):
    a = arrays
    return LP(int(c.rows), int(c.cols), a["col_starts"], a["row_index"], a["values"],
              a["col_cost"], a["col_lower"], a["col_upper"], a["row_lower"], a["row_upper"],
              sense, 0.0, a["x0"], a["lam"], float(c.fstar), name)


def planted_uniform(m: int, n: int, k: int = 5, seed: int = 1) -> LP:
    lib = _load()
    nnz = lib.lpgen_planted_uniform_nnz(m, n, k)
    arrays, c = _alloc(m, n, nnz)
    if lib.lpgen_planted_uniform(m, n, k, seed, ctypes.byref(c)) != 0:
        raise ValueError(f"planted_uniform: bad shape m={m} n={n} k={k}")
    return _finish(arrays, c, f"planted_uniform_{m}x{n}_k{k}_s{seed}")


def planted_blocks(blocks: int, rows_per_block: int, cols_per_block: int, k: int = 9,
                   seed: int = 1) -> LP:
    lib = _load()
    nnz = lib.lpgen_planted_blocks_nnz(blocks, rows_per_block, cols_per_block, k)
    m, n = blocks * rows_per_block, blocks * cols_per_block
    arrays, c = _alloc(m, n, nnz)
    if lib.lpgen_planted_blocks(blocks, rows_per_block, cols_per_block, k, seed,
                                ctypes.byref(c)) != 0:
        raise ValueError("planted_blocks: bad shape")
    return _finish(arrays, c, f"planted_blocks_{blocks}x{rows_per_block}x{cols_per_block}")


def planted_nondegenerate(m: int, n: int, k: int = 5, seed: int = 1) -> LP:
    """As planted_uniform with a unique, nondegenerate optimum (exactly m basic columns with
    a heavy diagonal in the basis): x* and y* are differentiable in the data."""
    lib = _load()
    nnz = lib.lpgen_planted_nondegenerate_nnz(m, n, k)
    arrays, c = _alloc(m, n, nnz)
    if lib.lpgen_planted_nondegenerate(m, n, k, seed, ctypes.byref(c)) != 0:
        raise ValueError("planted_nondegenerate: bad shape")
    return _finish(arrays, c, f"planted_nondegenerate_{m}x{n}")


def planted_zipf(m: int, n: int, target_nnz: int, exponent: float = 1.5, min_len: int = 2,
                 max_len: int = 100000, seed: int = 1) -> LP:
    """Load-balance stress: Zipf row lengths (P(L) ~ L^-exponent, clipped to
    [min_len, max_len], scaled to about target_nnz in total), uniform columns, values of
    log-uniform magnitude over [1e-3, 1e3] with random sign, 0 <= x <= 10, equality rows.
    500,000 x 1,000,000 with target 3e7 is the headline stress case."""
    lib = _load()
    nnz = lib.lpgen_planted_zipf_nnz(m, n, target_nnz, exponent, min_len, max_len, seed)
    if nnz < 0:
        raise ValueError("planted_zipf: bad shape")
    arrays, c = _alloc(m, n, nnz)
    if lib.lpgen_planted_zipf(m, n, target_nnz, exponent, min_len, max_len, seed,
                              ctypes.byref(c)) != 0:
        raise ValueError("planted_zipf: bad shape or more than 2^31 nonzeros")
    return _finish(arrays, c, f"planted_zipf_{m}x{n}")


def planted_general(m: int, n: int, k: int = 4, seed: int = 1, maximize: bool = False,
                    free: bool = True) -> LP:
    """Mixed row and column kinds. With ``maximize`` the cost is negated and the sense set
    to maximise, so the optimum point is unchanged and the objective is ``-fstar``. With
    ``free=False`` there are no free rows or columns."""
    lib = _load()
    nnz = lib.lpgen_planted_general_nnz(m, n, k)
    arrays, c = _alloc(m, n, nnz)
    if lib.lpgen_planted_general(m, n, k, 0 if free else 3, seed, ctypes.byref(c)) != 0:
        raise ValueError("planted_general: bad shape")
    lp = _finish(arrays, c, f"planted_general_{m}x{n}_s{seed}")
    if maximize:
        lp.col_cost = -lp.col_cost
        lp.sense = -1.0
    return lp

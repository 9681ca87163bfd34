"""Host-side checks of what the batched engine reports, in FP64 on the CPU.

``farkas_share(lp, d)`` checks an infeasibility certificate returned by
``BatchEngine.ray`` (sankhya_gb300_batch_ray). For the LP ``rl <= A x <= ru, l <= x <= u``
and a dual direction ``d`` with ``r = A'd``:

    value = sum_j min over [l_j, u_j] of r_j x_j  -  sum_i max over [rl_i, ru_i] of d_i s_i.

Any feasible x has ``r'x = d'(A x) <= sum_i max d_i s_i`` and ``r'x >= sum_j min r_j x_j``,
so ``value <= 0``; a positive value proves that no feasible x exists. A term whose bound is
absent while its coefficient is nonzero makes the value ``-inf`` (no proof). The share
returned is the value over the sum of the terms' magnitudes, so rounding (about 1e-16 of
that sum) cannot make a feasible LP look infeasible unless the share is that small.

The sums are taken with ``math.fsum`` (exactly rounded), and ``A'd`` per column with
``math.fsum`` too, so the check does not depend on the device's summation order.
"""
from __future__ import annotations

import math

import numpy as np

_HUGE = 1e30  # at or above this magnitude a bound is absent (include/sankhya/types.hpp:88-96)


def _finite(b):
    return np.abs(b) < _HUGE


def farkas_share(lp, d) -> float:
    """The certificate's value over its terms' magnitude; > 0 proves ``lp`` infeasible."""
    d = np.asarray(d, dtype=np.float64)
    if d.shape != (lp.rows,):
        raise ValueError(f"a ray of {lp.rows} entries is expected, got {d.shape}")
    starts = np.asarray(lp.col_starts, dtype=np.int64)
    prods = np.asarray(lp.values, dtype=np.float64) * d[np.asarray(lp.row_index)]
    r = np.array([math.fsum(prods[starts[j]:starts[j + 1]]) for j in range(lp.cols)])
    terms = []
    # Columns: min over [l, u] of r x.
    lo, up = np.asarray(lp.col_lower, float), np.asarray(lp.col_upper, float)
    pos, neg = r > 0, r < 0
    if np.any(pos & ~_finite(lo)) or np.any(neg & ~_finite(up)):
        return -math.inf
    terms.append(r[pos] * lo[pos])
    terms.append(r[neg] * up[neg])
    # Rows: - max over [rl, ru] of d s.
    rl, ru = np.asarray(lp.row_lower, float), np.asarray(lp.row_upper, float)
    dp, dn = d > 0, d < 0
    if np.any(dp & ~_finite(ru)) or np.any(dn & ~_finite(rl)):
        return -math.inf
    terms.append(-d[dp] * ru[dp])
    terms.append(-d[dn] * rl[dn])
    allt = np.concatenate(terms)
    mag = math.fsum(np.abs(allt))
    if mag == 0.0:
        return -math.inf
    return math.fsum(allt) / mag

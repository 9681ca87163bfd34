"""The host check of infeasibility certificates (sankhya_gb300.certify), on the CPU.

A certificate for an infeasible LP must score positive; no direction may score positive on a
feasible LP; a direction that leans on an absent bound is no proof.
"""
import numpy as np

from sankhya_gb300 import certify, lpgen
from sankhya_gb300.model import from_dense

INF = np.inf


def test_known_certificates():
    # x1 + x2 = 5 with 0 <= x <= 1: d = -1 gives r = (-1, -1), min r x = -2, -max(d s) = 5.
    lp = from_dense([[1, 1]], [5], [5], [1, 1], col_upper=[1, 1])
    assert certify.farkas_share(lp, np.array([-1.0])) > 0.0
    assert certify.farkas_share(lp, np.array([1.0])) < 0.0
    # x1 - x2 >= 3, x1 + x2 <= 1, 0 <= x <= 2: d = (-1, 1) sums the rows to 2 x2 <= -2.
    lp = from_dense([[1, -1], [1, 1]], [3, -INF], [INF, 1], [1, 2], col_upper=[2, 2])
    share = certify.farkas_share(lp, np.array([-1.0, 1.0]))
    assert share > 0.0
    # The share is the value over the terms' magnitude: here (0 - (-3) - 1) / (0 + 3 + 1).
    assert abs(share - 0.5) < 1e-15


def test_feasible_lps_have_no_certificate():
    rng = np.random.default_rng(0)
    for seed in range(3):
        lp = lpgen.planted_uniform(30, 60, 4, seed=seed)
        for _ in range(50):
            d = rng.standard_normal(lp.rows)
            assert certify.farkas_share(lp, d) <= 1e-12


def test_absent_bounds_give_no_proof():
    # x free above: any direction that needs the upper bound proves nothing.
    lp = from_dense([[1, 1]], [5], [5], [1, 1], col_upper=[INF, 1])
    assert certify.farkas_share(lp, np.array([-1.0])) == -np.inf
    assert certify.farkas_share(lp, np.zeros(1)) == -np.inf

"""Generate tests/golden/reference_qp.json: the REFERENCE's own convex-QP engine
(sankhya::qp::solve_convex_qp, src/qp/qp_condat_vu.cpp, compiled from its sources into
oracle/_ref/ by `make -C oracle ref`) run on small QPs.

Each case stores the QP itself (the LP part and the Hessian's stored triangle, every double as
a hex float), the solve options, and the reference's status, iteration count, objective (hex)
and SHA-256 digests of its col_value / col_dual / row_dual. The cases are the convex QPs of the
reference's tests/unit/test_qp.cpp (hand-derived optima), seeded random convex QPs in both
senses, with and without rows, and runs cut by the iteration limit. Run from the repository
root:  python tests/golden/make_golden_qp.py
"""
import hashlib
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "sih-26_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
from sankhya_gb300.model import qp_from_dense, random_qp  # noqa: E402

INF = float("inf")

# (name, QP builder, options): the first six are tests/unit/test_qp.cpp's convex instances.
CASES = [
    ("separable", lambda: qp_from_dense([-2.0, -8.0], [0, 0], [INF, INF],
                                        [(0, 0, 2.0), (1, 1, 4.0)]),
     dict(tolerance=1e-10, iteration_limit=500000)),
    ("bound_cuts_off", lambda: qp_from_dense([-2.0, -8.0], [0, 0], [0.25, INF],
                                             [(0, 0, 2.0), (1, 1, 4.0)]),
     dict(tolerance=1e-10, iteration_limit=500000)),
    ("coupling_row", lambda: qp_from_dense([0.0, 0.0], [0, 0], [INF, INF],
                                           [(0, 0, 1.0), (1, 1, 1.0)], [[1.0, 1.0]], [2.0],
                                           [2.0]),
     dict(tolerance=1e-10, iteration_limit=500000)),
    ("off_diagonal_twice", lambda: qp_from_dense([-4.0, -4.0], [0, 0], [INF, INF],
                                                 [(0, 0, 2.0), (1, 0, 1.0), (1, 1, 2.0)]),
     dict(tolerance=1e-10, iteration_limit=500000)),
    ("maximisation", lambda: qp_from_dense([2.0], [0], [INF], [(0, 0, -1.0)], sense=-1.0),
     dict(tolerance=1e-10, iteration_limit=500000)),
    ("singular_semidefinite", lambda: qp_from_dense([-2.0, -2.0], [0, 0], [10.0, 10.0],
                                                    [(0, 0, 1.0), (1, 0, 1.0), (1, 1, 1.0)]),
     dict(tolerance=1e-9, iteration_limit=500000)),
    ("random_min", lambda: random_qp(11, 30, 60), dict(tolerance=1e-8)),
    ("random_max", lambda: random_qp(12, 40, 70, maximise=True), dict(tolerance=1e-8)),
    ("random_wide_band", lambda: random_qp(13, 25, 80, per_column=6, hessian_band=5),
     dict(tolerance=1e-7)),
    ("random_no_rows", lambda: random_qp(14, 0, 50), dict(tolerance=1e-9)),
    ("random_cut_at_777", lambda: random_qp(15, 50, 90), dict(tolerance=1e-12,
                                                              iteration_limit=777)),
    ("random_seed_7", lambda: random_qp(16, 30, 60), dict(tolerance=1e-8, random_seed=7)),
]


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def hexes(a):
    return [float(v).hex() for v in np.asarray(a, dtype=np.float64)]


def encode(qp):
    lp = qp.lp
    return {"rows": lp.rows, "cols": lp.cols, "sense": lp.sense,
            "objective_offset": float(lp.objective_offset).hex(),
            "col_starts": [int(v) for v in lp.col_starts],
            "row_index": [int(v) for v in lp.row_index], "values": hexes(lp.values),
            "col_cost": hexes(lp.col_cost), "col_lower": hexes(lp.col_lower),
            "col_upper": hexes(lp.col_upper), "row_lower": hexes(lp.row_lower),
            "row_upper": hexes(lp.row_upper),
            "hessian_starts": [int(v) for v in qp.hessian_starts],
            "hessian_index": [int(v) for v in qp.hessian_index],
            "hessian_values": hexes(qp.hessian_values)}


def main():
    pyoracle.build(reference=True)
    if not pyoracle.reference_available():
        sys.exit("the reference library is not built (no reference tree)")
    ref = pyoracle.Oracle(reference=True)
    cases = []
    for name, make, options in CASES:
        qp = make()
        s = ref.solve_qp(qp, **options)
        cases.append({"name": name, "qp": encode(qp), "options": options,
                      "status": s.status_name, "iterations": s.iterations,
                      "objective": float(s.objective).hex(),
                      "col_value_sha256": digest(s.col_value),
                      "col_dual_sha256": digest(s.col_dual),
                      "row_dual_sha256": digest(s.row_dual)})
        print(f"{name}: {s.status_name}, {s.iterations} iterations, objective {s.objective!r}")
    with open(os.path.join(ROOT, "tests", "golden", "reference_qp.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden_qp.py",
                   "engine": "sankhya::qp::solve_convex_qp (src/qp/qp_condat_vu.cpp), the "
                             "reference's own sources built by `make -C oracle ref`",
                   "cases": cases}, f, indent=1)


if __name__ == "__main__":
    main()

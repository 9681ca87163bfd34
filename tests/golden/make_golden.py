"""Generate tests/golden/reference_pdhg.json: the REFERENCE's own PDHG (compiled from its
sources into oracle/_ref/ by `make -C oracle ref`) run on seeded synthetic instances.

Each case records the generator call that rebuilds the instance bit-for-bit (lpgen.c uses
IEEE basic operations only) with a SHA-256 of its arrays, the solve options, and the
reference's status, iteration and restart counts, objective (as a hex float), dual bound and
SHA-256 digests of the returned col_value / col_dual / row_dual. Run from the repository
root:  python tests/golden/make_golden.py
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
from sankhya_gb300 import build, lpgen  # noqa: E402

CASES = [
    ("planted_uniform", dict(m=200, n=500, k=5, seed=3), dict(tolerance=1e-8)),
    ("planted_uniform", dict(m=2000, n=5000, k=5, seed=1), dict(tolerance=1e-8)),
    ("planted_uniform", dict(m=100, n=250, k=5, seed=9), dict(tolerance=1e-6, stop_at_request=True)),
    ("planted_uniform", dict(m=100, n=250, k=5, seed=9),
     dict(tolerance=1e-8, restart=False, iteration_limit=3000)),
    ("planted_blocks", dict(blocks=8, rows_per_block=100, cols_per_block=200, k=9, seed=4),
     dict(tolerance=1e-8)),
    ("planted_general", dict(m=30, n=45, k=3, seed=100, free=False), dict(tolerance=1e-6)),
    ("planted_general", dict(m=30, n=45, k=3, seed=101, maximize=True, free=False),
     dict(tolerance=1e-6)),
    ("planted_general", dict(m=40, n=60, k=3, seed=2, free=True),
     dict(tolerance=1e-8, iteration_limit=20000)),
    ("planted_uniform", dict(m=300, n=700, k=5, seed=5), dict(tolerance=1e-12, iteration_limit=100)),
]


def make(gen, args):
    return getattr(lpgen, gen)(**args)


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def instance_digest(lp):
    return digest(lp.col_starts, lp.row_index, lp.values, lp.col_cost, lp.col_lower,
                  lp.col_upper, lp.row_lower, lp.row_upper)


def main():
    build.build_lpgen()
    pyoracle.build(reference=True)
    if not pyoracle.reference_available():
        raise SystemExit("the reference library is not built (needs the reference tree)")
    ref = pyoracle.Oracle(reference=True)
    out = []
    for gen, args, opts in CASES:
        lp = make(gen, args)
        s = ref.solve(lp, **opts)
        out.append(dict(
            generator=gen, args=args, options=opts, instance_sha256=instance_digest(lp),
            status=s.status_name, iterations=int(s.iterations), restarts=int(s.restarts),
            objective=float(s.objective).hex(), objective_float=float(s.objective),
            dual_bound=float(s.dual_bound).hex(),
            col_value_sha256=digest(s.col_value), col_dual_sha256=digest(s.col_dual),
            row_dual_sha256=digest(s.row_dual), message=s.message))
        print(gen, args, s.status_name, s.iterations, s.objective)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_pdhg.json")
    with open(path, "w") as f:
        json.dump({"source": "reference PDHG (src/pdhg/pdhg.cpp) compiled from its own sources",
                   "cases": out}, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()

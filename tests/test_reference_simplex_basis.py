"""The adjoint's reference gradient, built from the reference simplex's optimal basis.

The GPU adjoint tests (tests/test_gpu_adjoint.py) compare the engine's gradients with
gradients built from the planted basis of each nondegenerate LP: B = the columns strictly
inside their box. The requirement is a comparison with the gradient built from the optimal
basis that the REFERENCE's simplex finds. Here, on the CPU, the reference's own dual simplex
solves the same LPs, through its own Python package (bindings/python/sankhya) on a build of
its core. Its optimal basis must be the planted one, with x* and y* the planted point. The
gradient built from its basis must then equal the planted-basis gradient that the GPU tests
hold the engine to. Needs the reference tree (skips without it).
"""
import os
import subprocess
import sys
import textwrap

import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The LPs of test_gpu_adjoint.test_adjoint_matches_basis_solves (m, seed), and one larger.
CASES = [(m, 900 + m + s) for m in (30, 80, 150) for s in range(2)] + [(1000, 7)]


def test_reference_simplex_basis_gives_the_planted_gradient(reference_core_library):
    script = textwrap.dedent(f"""
        import sys
        sys.path[:0] = [{os.path.join(pyoracle.REFERENCE_TREE, "bindings", "python")!r},
                        {os.path.join(ROOT, "sih-26_gb300")!r}]
        import numpy as np
        import sankhya
        from sankhya_gb300 import lpgen

        def gradients(A, c, B, at_lower, at_upper, x, y, gx, gy, gf):
            # Implicit differentiation at a nondegenerate vertex with basis B and nonbasic
            # columns at_lower / at_upper (all rows are equalities): p = A_B^-T g_x[B],
            # q = A_B^-1 g_y.
            d = c - A.T @ y
            p = np.linalg.solve(A[:, B].T, gx[B])
            q = np.linalg.solve(A[:, B], gy)
            dc = gf * x.copy()
            dc[B] += q
            db = p + gf * y
            dbound = gx - A.T @ p + gf * d
            return dc, db, np.where(at_lower, dbound, 0.0), np.where(at_upper, dbound, 0.0)

        for m, seed in {CASES!r}:
            lp = lpgen.planted_nondegenerate(m, 2 * m, 5, seed=seed)
            A = np.zeros((lp.rows, lp.cols))
            model = sankhya.Model()
            for j in range(lp.cols):
                model.add_column(cost=lp.col_cost[j], lower=lp.col_lower[j],
                                 upper=lp.col_upper[j])
            rows = [dict() for _ in range(lp.rows)]
            for j in range(lp.cols):
                for k in range(lp.col_starts[j], lp.col_starts[j + 1]):
                    rows[lp.row_index[k]][j] = float(lp.values[k])
                    A[lp.row_index[k], j] = lp.values[k]
            for i in range(lp.rows):
                model.add_row(rows[i], lower=lp.row_lower[i], upper=lp.row_upper[i])
            r = model.solve(algorithm="dual-simplex", log_to_console=False)
            assert r.status == "optimal", (m, seed, r.status, r.message)
            basis = np.array(r.col_statuses) == "basic"
            planted = (lp.x0 > lp.col_lower) & (lp.x0 < lp.col_upper)
            assert basis.sum() == m and set(r.row_statuses) == {{"fixed"}}, (m, seed)
            assert np.array_equal(basis, planted), (m, seed, "basis differs")
            x, y = np.array(r.x), np.array(r.row_duals)
            assert np.abs(x - lp.x0).max() <= 1e-9 and np.abs(y - lp.lam).max() <= 1e-9
            assert abs(r.objective - lp.fstar) <= 1e-9 * max(1.0, abs(lp.fstar))
            rng = np.random.default_rng(seed)
            gx, gy = rng.standard_normal(lp.cols), rng.standard_normal(lp.rows)
            status = np.array(r.col_statuses)
            ref = gradients(A, lp.col_cost, basis, status == "at_lower", status == "at_upper",
                            x, y, gx, gy, 1.0)
            want = gradients(A, lp.col_cost, planted, ~planted & (lp.x0 <= lp.col_lower),
                             ~planted & (lp.x0 >= lp.col_upper), lp.x0, lp.lam, gx, gy, 1.0)
            for a, b in zip(ref, want):
                assert np.all(np.abs(a - b) <= 1e-9 * np.maximum(1.0, np.abs(b))), (m, seed)
            print(m, seed, "simplex basis = planted basis", flush=True)
        print("OK")
        """)
    env = dict(os.environ, SANKHYA_LIBRARY=reference_core_library)
    run = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                         timeout=900, env=env)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-3000:]
    assert run.stdout.strip().endswith("OK"), run.stdout

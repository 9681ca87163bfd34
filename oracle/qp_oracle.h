/*
 * qp_oracle.h -- CPU restatement of SANKHYA's convex-QP engine (Condat-Vu), used ONLY as a
 * checker.
 *
 * TEST INFRASTRUCTURE. Only tests/ and bench.py's CPU legs load this code (it is part of
 * liboracle.so with pdhg_oracle.c). The GPU QP engine never calls it and never falls back
 * to it.
 *
 * Each function restates one reference function, cited by file:line inside the reference
 * project (thegoodengineer/sih-26):
 *   orc_qp_spectral_norm   src/qp/qp_condat_vu.cpp:74-103   (||A||, 20 power steps)
 *   orc_qp_hessian_norm    src/qp/qp_condat_vu.cpp:105-143  (|lambda| of Q, 20 power steps)
 *   orc_qp_hessian_multiply src/qp/qp_condat_vu.cpp:145-160 (Q x from the stored triangle)
 *   orc_qp_objective       src/core/model.cpp:101-125       (Model::evaluate_objective)
 *   orc_solve_qp           src/qp/qp_condat_vu.cpp:164-362  (the whole engine, after its
 *                                                            convexity gate)
 * The convexity gate itself (src/qp/convexity.cpp, a sparse LDL^T) is not restated: the
 * callers that need it run the reference's own.
 *
 * Pinning: tests/test_qp_oracle.py runs this code and the reference's solve_convex_qp
 * (compiled from its own sources by oracle/Makefile into oracle/_ref/) on the same QPs and
 * requires identical statuses and iteration counts and bit-identical points; it also holds
 * the restatement to the hand-derived optima of the reference's tests/unit/test_qp.cpp.
 * Built with -ffp-contract=off, like pdhg_oracle.c.
 */
#ifndef SANKHYA_QP_ORACLE_H
#define SANKHYA_QP_ORACLE_H

#include <stdint.h>

#include "pdhg_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A convex QP in the reference Model's layout: the LP part (A, c, bounds, sense, offset) and
 * the Hessian Q as Model::hessian holds it (include/sankhya/model.hpp): a CSC matrix of
 * cols x cols whose entries are the lower triangle of the symmetric Q, so that the objective
 * is offset + c'x + 0.5 x'Qx. An off-diagonal entry (i, j) stands for Q_ij and Q_ji. */
typedef struct {
  orc_lp lp;
  const int32_t* hessian_starts; /* cols + 1, or NULL for no quadratic term */
  const int32_t* hessian_index;
  const double* hessian_values;
} orc_qp;

typedef struct {
  double tolerance;        /* qp_tolerance */
  int64_t iteration_limit; /* iteration_limit; < 0: the engine's ceiling of 1,000,000 */
  double time_limit;       /* seconds; <= 0 is a zero budget, >= 1e300 means none */
  int64_t random_seed;     /* random_seed */
} orc_qp_params;

typedef struct {
  int32_t status;  /* ORC_OPTIMAL, ORC_ITERATION_LIMIT or ORC_TIME_LIMIT */
  int32_t ceiling; /* 1 when the iteration limit was the engine's own ceiling */
  int64_t iterations;
  double primal_residual; /* at the last check (every 50 iterations); -1 before the first */
  double dual_residual;
  double norm_a, norm_q, tau, sigma;
  double objective; /* Model::evaluate_objective at the reported point */
  double solve_seconds;
} orc_qp_result;

double orc_qp_spectral_norm(int32_t rows, int32_t cols, const int32_t* col_starts,
                            const int32_t* row_index, const double* values, uint32_t seed);
double orc_qp_hessian_norm(const orc_qp* qp, uint32_t seed);
/* out = Q x (cols entries). */
void orc_qp_hessian_multiply(const orc_qp* qp, const double* x, double* out);
double orc_qp_objective(const orc_qp* qp, const double* x);

/* The engine after its convexity gate. col_value / col_dual (cols) and row_dual (rows) may be
 * NULL; they are filled as the reference fills Solution (src/qp/qp_condat_vu.cpp:343-353):
 * col_value = x, row_dual = -sense * y, col_dual = c + Qx + sense * A'y. */
int32_t orc_solve_qp(const orc_qp* qp, const orc_qp_params* params, orc_qp_result* result,
                     double* col_value, double* col_dual, double* row_dual);

#ifdef __cplusplus
}
#endif
#endif

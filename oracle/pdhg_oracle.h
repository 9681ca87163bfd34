/*
 * pdhg_oracle.h -- CPU restatement of SANKHYA's restarted PDHG, used ONLY as a checker.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load this library. The GPU engine never calls it and never falls back to it.
 *
 * Every function restates one reference function, cited by file:line inside the reference
 * project (thegoodengineer/sih-26):
 *   orc_multiply            src/la/sparse.cpp:232-242,261-264   (A x, column scatter)
 *   orc_transpose_multiply  src/la/sparse.cpp:244-259,266-269   (A^T y, column gather)
 *   orc_build_scaling       src/la/scaling.cpp:14-159           (Ruiz x10 + Pock-Chambolle)
 *   orc_spectral_norm       src/la/scaling.cpp:161-194          (power iteration on A^T A)
 *   orc_evaluate            src/pdhg/pdhg_evaluate.cpp:19-139   (unscaled residuals)
 *   orc_solve_pdhg          src/pdhg/pdhg.cpp:76-568            (the whole engine)
 *
 * Pinning: tests/test_oracle_vs_reference.py runs this library and the reference itself
 * (compiled from its own sources by oracle/Makefile into oracle/_ref/) on the same inputs
 * and requires identical iteration counts, restarts and bit-identical objectives; the
 * committed fixtures under tests/golden/ carry the reference's outputs to machines where
 * the reference sources are absent.
 *
 * Built with -ffp-contract=off so that no multiply-add is fused on either x86-64 or
 * aarch64, which keeps the arithmetic identical to the reference's x86-64 build.
 */
#ifndef SANKHYA_PDHG_ORACLE_H
#define SANKHYA_PDHG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status values: the reference's C API codes, include/sankhya/sankhya.h:53-69. */
enum {
  ORC_NOT_SOLVED = 0,
  ORC_OPTIMAL = 1,
  ORC_FEASIBLE = 2,
  ORC_INFEASIBLE = 3,
  ORC_ITERATION_LIMIT = 5,
  ORC_TIME_LIMIT = 6,
  ORC_NUMERICAL_ERROR = 8,
  ORC_MODEL_ERROR = 9,
  ORC_INTERRUPTED = 11
};

/* An LP in the reference Model's layout (include/sankhya/model.hpp:123-170): CSC with
 * int32 indices and ascending row indices inside each column, FP64 values, two-sided rows
 * rl <= Ax <= ru and columns l <= x <= u; +-inf (or |v| >= 1e30) means "no bound". */
typedef struct {
  int32_t rows;
  int32_t cols;
  const int32_t* col_starts; /* cols + 1 */
  const int32_t* row_index;  /* nnz */
  const double* values;      /* nnz */
  const double* col_cost;
  const double* col_lower;
  const double* col_upper;
  const double* row_lower;
  const double* row_upper;
  double sense; /* +1 minimise, -1 maximise (Model::sense_multiplier) */
  double objective_offset;
} orc_lp;

typedef struct {
  double tolerance;        /* pdhg_tolerance */
  int64_t iteration_limit; /* iteration_limit; < 0 means the engine's own 1e6 ceiling */
  double time_limit;       /* seconds; <= 0 is a zero budget, >= 1e300 means none (the
                              reference's kNoLimit is DBL_MAX, src/util/options.cpp:30) */
  int32_t restart;         /* pdhg_restart */
  int32_t stop_at_request; /* pdhg_stop_at_request */
  int64_t random_seed;     /* random_seed */
} orc_params;

/* Mirrors sankhya::pdhg::Residuals (src/pdhg/pdhg_evaluate.hpp:19-70). */
typedef struct {
  double primal, dual, gap;
  double primal_objective, dual_objective;
  double absolute_primal, absolute_dual;
  double gap_as_verified, complementarity;
} orc_residuals;

typedef struct {
  int32_t status;
  int32_t pad;
  int64_t iterations;
  int64_t restarts;
  double objective;  /* Model::evaluate_objective at the reported point */
  double dual_bound; /* only when optimal, else -+inf */
  orc_residuals final_residuals;
  double spectral_norm;
  double scaled_min_abs;
  double scaled_max_abs;
  double solve_seconds;
  int64_t evaluations;
} orc_result;

/* y = A x (column scatter that skips zero x_j). */
void orc_multiply(int32_t rows, int32_t cols, const int32_t* col_starts, const int32_t* row_index,
                  const double* values, const double* x, double* y);
/* y = A^T x (per-column gather). */
void orc_transpose_multiply(int32_t rows, int32_t cols, const int32_t* col_starts,
                            const int32_t* row_index, const double* values, const double* x,
                            double* y);

/* The scaled problem of build_scaling: Ahat values (CSC order, same pattern), Dr, Dc, and the
 * scaled cost / bounds. min_space_cost is sense * col_cost. */
void orc_build_scaling(const orc_lp* lp, const double* min_space_cost, int32_t ruiz_iterations,
                       double* scaled_values, double* row_scale, double* col_scale,
                       double* scaled_cost, double* scaled_col_lower, double* scaled_col_upper,
                       double* scaled_row_lower, double* scaled_row_upper, double* min_abs,
                       double* max_abs);

double orc_spectral_norm(int32_t rows, int32_t cols, const int32_t* col_starts,
                         const int32_t* row_index, const double* values, int32_t iterations,
                         uint32_t seed);

/* Residuals of the unscaled candidate (x, y); activity (m) and reduced (n) are outputs. */
orc_residuals orc_evaluate(const orc_lp* lp, const double* x, const double* y, double* activity,
                           double* reduced);

/* The whole reference engine. col_value/col_dual (n) and row_dual (m) may be NULL. */
int32_t orc_solve_pdhg(const orc_lp* lp, const orc_params* params, orc_result* result,
                       double* col_value, double* col_dual, double* row_dual);

/* The first `count` doubles of the std::mt19937 + uniform_real_distribution(-1, 1) stream
 * the power iteration starts from (src/la/scaling.cpp:168-171). */
void orc_power_start(uint32_t seed, int32_t count, double* out);

#ifdef __cplusplus
}
#endif
#endif

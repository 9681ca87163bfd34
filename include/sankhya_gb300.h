/*
 * sankhya_gb300.h -- the C ABI of the GB300-native restarted-PDHG engine.
 *
 * This is the boundary SANKHYA's PDHG path binds to. It replaces the reference's CUDA
 * engine behind the unchanged C++ seam
 *     Solution sankhya::gpu::solve_pdhg_gpu(const Model&, const Options&, Logger&,
 *                                           SolveControl*)          (src/gpu/pdhg_gpu.hpp:19-20)
 * whose only caller is src/core/solve.cpp:802. The seam (sih-26_gb300/seam/pdhg_gpu.cpp)
 * converts the Model / Options into the plain structs below and calls these functions.
 *
 * Conventions (the reference's C API, include/sankhya/sankhya.h:36-50 and
 * src/api/c_api.cpp:39,134-150): every function returns an int status, 0 on success; the
 * message of the last failure on this thread is sankhya_gb300_last_error(). Nothing throws
 * across this boundary. All pointers are HOST pointers; the engine copies what it needs to
 * the device and owns every device allocation. There is no CPU fallback: with no usable
 * GPU the calls fail with SANKHYA_GB300_ERROR_DEVICE.
 *
 * Threads: an engine handle holds one LP (or one batch) and its device state, so calls on
 * one handle must not overlap; a caller that shares a handle between threads serialises
 * them, as the seam does for its one engine. Different handles are independent, except that
 * the kernel-launch count the results report is kept per process.
 */
#ifndef SANKHYA_GB300_H
#define SANKHYA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SGB_API __attribute__((visibility("default")))
#else
#define SGB_API
#endif

/* Return codes: sankhya_status (include/sankhya/sankhya.h:42-50) plus one for the device. */
enum {
  SANKHYA_GB300_OK = 0,
  SANKHYA_GB300_ERROR_ARGUMENT = 1,
  SANKHYA_GB300_ERROR_MODEL = 3,
  SANKHYA_GB300_ERROR_OPTION = 4,
  SANKHYA_GB300_ERROR_MEMORY = 5,
  SANKHYA_GB300_ERROR_INTERNAL = 6,
  SANKHYA_GB300_ERROR_DEVICE = 7 /* no usable CUDA device, or a CUDA call failed */
};

/* Solve status: the values of sankhya_solve_status (include/sankhya/sankhya.h:53-69). */
enum {
  SANKHYA_GB300_NOT_SOLVED = 0,
  SANKHYA_GB300_OPTIMAL = 1,
  SANKHYA_GB300_FEASIBLE = 2,
  SANKHYA_GB300_INFEASIBLE = 3,
  SANKHYA_GB300_ITERATION_LIMIT = 5,
  SANKHYA_GB300_TIME_LIMIT = 6,
  SANKHYA_GB300_NUMERICAL_ERROR = 8,
  SANKHYA_GB300_MODEL_ERROR = 9,
  SANKHYA_GB300_INTERRUPTED = 11
};

/* Arithmetic of the PDHG iterations (new option row `pdhg_precision`). */
enum {
  SANKHYA_GB300_FP64 = 0,  /* the reference's method, FP64 throughout */
  SANKHYA_GB300_MIXED = 1  /* FP32 iterates / values / SpMV, FP64 KKT and refinement */
};

/* When the loop stops (new option row `pdhg_stop_rule`). STANDARD is the reference's test
 * (src/pdhg/pdhg.cpp:424-425): the request (relative primal, dual, gap <= tolerance and
 * absolute primal <= 1e-7) and, unless stop_at_request, the absolute project standard.
 * RELATIVE stops as soon as the relative KKT error max(primal, dual, gap) <= tolerance.
 * Either way the status is `optimal` only if the reported point meets the project
 * standard, else `feasible` (src/pdhg/pdhg.cpp:515-536). */
enum {
  SANKHYA_GB300_STOP_STANDARD = 0,
  SANKHYA_GB300_STOP_RELATIVE = 1
};

/* An LP in sankhya::Model's layout (include/sankhya/model.hpp:123-170): CSC, int32 indices
 * ascending inside each column, FP64 values, rows rl <= Ax <= ru, columns l <= x <= u; an
 * infinite bound is +-inf or any magnitude >= 1e30. */
typedef struct sankhya_gb300_lp {
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
  double sense;            /* +1 minimise, -1 maximise (Model::sense_multiplier) */
  double objective_offset; /* Model::objective_offset */
} sankhya_gb300_lp;

/* One iteration-table row, the arguments of Logger::iteration (src/pdhg/pdhg.cpp:399). */
typedef void (*sankhya_gb300_log_fn)(void* user, long long iteration, double objective,
                                     double primal, double dual, double seconds);

/* Polled at every status snapshot; a nonzero return interrupts the solve (the reference's
 * StopController::should_stop, src/core/stop_controller.hpp:36-75: SolveControl::interrupt()
 * or a progress callback asking to stop). */
typedef int (*sankhya_gb300_poll_fn)(void* user, long long iteration, double objective);

/* The PDHG option rows (src/util/options.cpp) plus the engine's own. */
typedef struct sankhya_gb300_params {
  double tolerance;          /* pdhg_tolerance */
  int64_t iteration_limit;   /* iteration_limit; < 0: the engine's 1e6 ceiling (pdhg.cpp:124) */
  double time_limit;         /* time_limit in seconds; >= 1e300 means none */
  int32_t restart;           /* pdhg_restart */
  int32_t stop_at_request;   /* pdhg_stop_at_request */
  int64_t random_seed;       /* random_seed (power-iteration start, scaling.cpp:168) */
  int32_t precision;         /* SANKHYA_GB300_FP64 or SANKHYA_GB300_MIXED */
  int32_t steps_per_poll;    /* attempted steps per CUDA-graph launch; 0 = default */
  int32_t stop_rule;         /* SANKHYA_GB300_STOP_STANDARD or SANKHYA_GB300_STOP_RELATIVE */
  int32_t reserved;
  const volatile int32_t* interrupt; /* an interrupt flag, polled; may be NULL */
  sankhya_gb300_log_fn log;  /* may be NULL */
  void* log_user;
  sankhya_gb300_poll_fn poll; /* may be NULL */
  void* poll_user;
} sankhya_gb300_params;

/* sankhya::pdhg::Residuals (src/pdhg/pdhg_evaluate.hpp:19-70). */
typedef struct sankhya_gb300_residuals {
  double primal, dual, gap;
  double primal_objective, dual_objective;
  double absolute_primal, absolute_dual;
  double gap_as_verified, complementarity;
} sankhya_gb300_residuals;

typedef struct sankhya_gb300_result {
  int32_t status;        /* SANKHYA_GB300_OPTIMAL, ... */
  int32_t converged;     /* the loop met its stopping test */
  int64_t iterations;    /* accepted steps (Solution::iterations) */
  int64_t attempts;      /* attempted steps, accepted or not */
  int64_t restarts;
  int64_t evaluations;
  int64_t refinements;   /* mixed precision: refinement rounds */
  double objective;      /* objective_offset + col_cost . x at the reported point */
  double dual_bound;     /* only when optimal, else -+inf (pdhg.cpp:553-557) */
  sankhya_gb300_residuals final_residuals;
  double spectral_norm;
  double scaled_min_abs, scaled_max_abs;
  double setup_seconds;  /* scaling + power iteration on the device */
  double loop_seconds;   /* the PDHG loop */
  double solve_seconds;  /* the whole solve call, host clock */
  double device_seconds; /* the whole solve, CUDA events on the engine's stream */
  int64_t kernel_launches; /* engine kernels launched by this solve (graph nodes included) */
  /* Share of the nonzeros whose gathered element the step pass of this precision reads from
   * a staged shared-memory window rather than global memory: [0] column pass, [1] row pass. */
  double staged_fraction[2];
  char message[512];
} sankhya_gb300_result;

typedef struct sankhya_gb300_pdhg sankhya_gb300_pdhg; /* opaque engine handle */

/* Message of the last failure on the calling thread ("" if none). c_api.cpp:39. */
SGB_API const char* sankhya_gb300_last_error(void);

/* Device probes: src/gpu/device.hpp:19-29 (device_available, device_free_memory,
 * device_compute_capability). description may be NULL. */
SGB_API int sankhya_gb300_device_available(char* description, int32_t capacity);
SGB_API int sankhya_gb300_device_free_memory(size_t* free_bytes, size_t* total_bytes);
SGB_API int sankhya_gb300_device_compute_capability(int32_t* major, int32_t* minor);

/* Device bytes the engine allocates for an LP of this size (replaces
 * estimate_pdhg_gpu_memory, src/gpu/gpu_memory.hpp:35-44). Pure arithmetic. */
SGB_API size_t sankhya_gb300_estimate_memory(int32_t rows, int32_t cols, int64_t nonzeros,
                                             int32_t precision);

/* Create / destroy an engine on a device (the state GpuState held, src/gpu/pdhg_gpu.cu:201). */
SGB_API int sankhya_gb300_pdhg_create(int32_t device, sankhya_gb300_pdhg** out);
SGB_API int sankhya_gb300_pdhg_destroy(sankhya_gb300_pdhg* engine);

/* Copy an LP to the device: CSC and a CSR copy, unscaled values kept for the evaluation.
 * Fails with SANKHYA_GB300_ERROR_MODEL on the numeric defects Model::validate rejects
 * (src/core/model.cpp:127-240): a matrix value that is not finite, a NaN bound, a crossed
 * bound, a NaN cost, a NaN objective offset; and on a CSC structure that is not well formed
 * (column starts not from 0 or not monotone, a row index out of range, row indices not
 * strictly ascending in a column). It also refuses an INFINITE cost, which Model::validate
 * lets through: on such an LP the reference PDHG returns a NaN objective at its iteration
 * limit, or never ends when the column can move towards the infinite cost. Negative sizes
 * or null column starts fail with SANKHYA_GB300_ERROR_ARGUMENT. */
SGB_API int sankhya_gb300_pdhg_load(sankhya_gb300_pdhg* engine, const sankhya_gb300_lp* lp);

/* Solve the loaded LP: device preconditioning (src/la/scaling.cpp:111-194) and the restarted
 * PDHG loop (src/pdhg/pdhg.cpp:76-568) with every iterate resident on the device. */
SGB_API int sankhya_gb300_pdhg_solve(sankhya_gb300_pdhg* engine,
                                     const sankhya_gb300_params* params,
                                     sankhya_gb300_result* result);

/* The reported point of the last solve, filled as solve_pdhg fills Solution
 * (src/pdhg/pdhg.cpp:487-501): col_value = x, col_dual = sense * (c + A^T y),
 * row_dual = sense * (-y). Any pointer may be NULL. */
SGB_API int sankhya_gb300_pdhg_solution(sankhya_gb300_pdhg* engine, double* col_value,
                                        double* col_dual, double* row_dual);

/* Parity hooks for tests: the device preconditioning of the loaded LP (Dr, Dc, the scaled CSC
 * values and the spectral-norm estimate), and one product with the loaded matrix:
 * op 0 = A x (x has cols entries), op 1 = A^T y (y has rows entries); scaled != 0 uses the
 * scaled matrix of the last preconditioning. */
SGB_API int sankhya_gb300_pdhg_scaling(sankhya_gb300_pdhg* engine, int64_t random_seed,
                                       double* row_scale, double* col_scale,
                                       double* scaled_values, double* spectral_norm);
SGB_API int sankhya_gb300_pdhg_spmv(sankhya_gb300_pdhg* engine, int32_t op, int32_t scaled,
                                    const double* in, double* out);

/* The same product on DEVICE buffers, allocating nothing. It has no reference counterpart:
 * the reference's products (src/la/sparse.cpp:232-259) are host-side only. It is for callers
 * that hold their vectors in device memory and may not allocate: a device allocation
 * synchronises the whole GPU and fails when a caching allocator has already reserved the
 * memory. `device_in` (cols entries for op 0, rows for op 1) and `device_out` are device
 * pointers; the work is enqueued on `stream` (a cudaStream_t; NULL = the engine's stream)
 * and the call returns without waiting for it. Its only scratch is a fixed device array of
 * SANKHYA_GB300_NOALLOC_MAX_CHUNKS partial sums (one per 2048 entries of each row longer than
 * 2048) plus a counter, 128 KiB that every GPU which loads this library keeps until the
 * process exits; a matrix that needs more slots is refused with
 * SANKHYA_GB300_ERROR_ARGUMENT. The first call on a device sets that scratch up (finds it and
 * clears the counter, waiting for the stream) and must come before any stream capture.
 * Calls on one device share the scratch: calls that overlap in time race, so order them
 * (one stream, or events between streams). The scratch's device address is looked up once
 * per device index and kept for the life of the process: after cudaDeviceReset (or anything
 * else that destroys the device's primary context) the kept address is stale, so a process
 * that resets a device must not call this entry point on it again. The call does not wait
 * for the product, so it cannot report a failure of the product itself: if a bounded wait in
 * the product gives up (a copy that never lands), the rows it could not finish are set to
 * NaN instead of being left with a result that looks valid. */
#define SANKHYA_GB300_NOALLOC_MAX_CHUNKS 16384
SGB_API int sankhya_gb300_pdhg_spmv_noalloc(sankhya_gb300_pdhg* engine, int32_t op,
                                            int32_t scaled, const double* device_in,
                                            double* device_out, void* stream);

/* Measurement hook: time `reps` attempted PDHG steps on the state the last solve left,
 * each kernel bracketed by CUDA events on the engine's stream. ms[0] = mean duration of the
 * primal (column) pass, ms[1] = mean duration of the dual (row) pass, in milliseconds. The
 * solve's results are restored afterwards. */
SGB_API int sankhya_gb300_pdhg_time_kernels(sankhya_gb300_pdhg* engine, int32_t reps,
                                            double* ms);

/* ---- Batched solves ------------------------------------------------------------------------
 * Many LPs solved together on one device, each by one thread block in one persistent launch,
 * with its own step size, primal weight, restart state and stopping test: the reference's
 * PDHG (src/pdhg/pdhg.cpp), per LP, as solve_pdhg runs it. No reference counterpart: it is
 * the batched engine of the branch-and-bound node relaxations (the reference solves those
 * one at a time, src/mip/branch_and_bound_node.cpp) and of many small LPs. LPs whose
 * col_starts / row_index / values pointers and sizes are equal share one device copy of the
 * matrix (scaled and norm-estimated once). An LP whose dual iterate drifts along a Farkas ray
 * is reported SANKHYA_GB300_INFEASIBLE. Options: tolerance, iteration_limit, restart,
 * stop_at_request, random_seed, stop_rule and precision (SANKHYA_GB300_MIXED runs the mixed
 * method per LP: FP32 iterations on FP64 refinement rounds); time_limit, interrupt, log and
 * poll are not used. */
typedef struct sankhya_gb300_batch sankhya_gb300_batch;

typedef struct sankhya_gb300_batch_item {
  int32_t status; /* SANKHYA_GB300_OPTIMAL, FEASIBLE, INFEASIBLE or ITERATION_LIMIT */
  int32_t converged;
  int64_t iterations, attempts, restarts, evaluations;
  double objective;  /* objective_offset + col_cost . x at the reported point */
  double dual_bound; /* only when optimal, else -+inf */
  sankhya_gb300_residuals final_residuals;
  double spectral_norm;
  double farkas_value; /* infeasible: the certificate's value over its terms' magnitude */
  int64_t refinements; /* mixed precision: refinement rounds of this LP */
} sankhya_gb300_batch_item;

SGB_API int sankhya_gb300_batch_create(int32_t device, sankhya_gb300_batch** batch);
SGB_API int sankhya_gb300_batch_destroy(sankhya_gb300_batch* batch);
SGB_API int sankhya_gb300_batch_load(sankhya_gb300_batch* batch, int32_t count,
                                     const sankhya_gb300_lp* lps);
/* items has `count` entries; device_seconds (may be NULL) receives the solve's device time
 * (CUDA events around the two launches). */
SGB_API int sankhya_gb300_batch_solve(sankhya_gb300_batch* batch,
                                      const sankhya_gb300_params* params,
                                      sankhya_gb300_batch_item* items, double* device_seconds);
/* The schedule of the batch's next solves (no reference counterpart): `lanes` threads share a
 * row or column in the matrix passes (1, 2, 4, 8, 16 or 32) and each LP is solved by a block
 * of `threads` threads (128, 256 or 512). lanes = threads = 0 (the default) lets every solve
 * pick the schedule itself: before the solve it times each of 1, 2, 4 and 8 lanes at 128,
 * 256 and 512 threads for 200 steps on a sample of the batch (up to four LPs per SM, spread
 * over the LPs' sizes) and takes the fastest. Sums inside a row or column are taken in a
 * fixed order for a given schedule, so a fixed schedule gives bit-reproducible solves; an
 * autotuned one may pick differently from run to run. Anything else is
 * SANKHYA_GB300_ERROR_ARGUMENT. */
SGB_API int sankhya_gb300_batch_schedule(sankhya_gb300_batch* batch, int32_t lanes,
                                         int32_t threads);
/* The schedule the last solve ran with and the seconds its autotuning took (0 when the
 * schedule was set). Any pointer may be NULL. */
SGB_API int sankhya_gb300_batch_last_schedule(sankhya_gb300_batch* batch, int32_t* lanes,
                                              int32_t* threads, double* tune_seconds);
/* The reported point of LP `index`, as sankhya_gb300_pdhg_solution. */
SGB_API int sankhya_gb300_batch_solution(sankhya_gb300_batch* batch, int32_t index,
                                         double* col_value, double* col_dual,
                                         double* row_dual);
/* Replaces the reported point of LP `index` (after a solve) with the caller's, given as
 * sankhya_gb300_batch_solution returns it: a warm start for sankhya_gb300_batch_polish, which
 * reads the active sets from that point and re-solves them for the LP's own data. No
 * reference counterpart: the reference warm-starts a branch-and-bound node from its parent's
 * basis inside its simplex (src/mip/branch_and_bound_node.cpp); this is the same hand-over for
 * the batched engine, e.g. a child node polished from its parent's vertex. */
SGB_API int sankhya_gb300_batch_set_point(sankhya_gb300_batch* batch, int32_t index,
                                          const double* col_value, const double* col_dual,
                                          const double* row_dual);
/* The infeasibility certificate of LP `index` when the last solve reported it
 * SANKHYA_GB300_INFEASIBLE (no reference counterpart: the reference's PDHG reports no
 * infeasibility): `ray` (m entries) receives the dual direction d, in the LP's own units,
 * whose value
 *   sum_j min over [l_j, u_j] of (A'd)_j x_j  -  sum_i max over [rl_i, ru_i] of d_i s_i
 * is positive, which no feasible x allows (every term is finite for a certificate). For any
 * other status it holds the last direction tested, which proves nothing. */
SGB_API int sankhya_gb300_batch_ray(sankhya_gb300_batch* batch, int32_t index, double* ray);

/* Gradients through the last batch solve (no reference counterpart: the reference has no
 * differentiation). For L(x, y, f) at the optimum, with x = col_value, y = row_dual (the
 * derivative of f by a row bound) and f = objective, given per LP the upstream gradients
 * dl_dx[k] (cols), dl_dy[k] (rows) and dl_df[k], returns dL/dc, dL/d(row_lower),
 * dL/d(row_upper), dL/d(col_lower), dL/d(col_upper) by implicit differentiation of the
 * optimum: at the active set the PDHG fixed point reduces to two square linear systems with
 * the basis matrix A_RB, solved on the device on a compact copy of A_RB by preconditioned
 * conjugate gradients on its normal equations, with refinement passes. An equality row's
 * dL/db is dl_drl + dl_dru (only the side its multiplier's sign names is nonzero). Any
 * upstream pointer may be NULL (zero); any output pointer may be NULL. Minimisation and
 * maximisation LPs alike (the sense is folded as src/pdhg/pdhg.cpp:95-111 folds it). */
typedef struct sankhya_gb300_adjoint_info {
  int32_t status;      /* 0 ok, 1 degenerate optimum (|B| != |R|), 2 CG not converged */
  int32_t basic_cols;  /* |B| */
  int32_t active_rows; /* |R| */
  int32_t iterations[2];
  double residual[2];
} sankhya_gb300_adjoint_info;

/* Active-set polish of the last batch solve (no reference counterpart; it plays the part
 * of the reference's PDHG -> interior-point polish hand-off, src/core/solve.cpp:239-308, for
 * nondegenerate LPs): at each converged LP's active sets, x_B and the multipliers are
 * re-solved from the basis matrix A_RB (the adjoint's square solves, started from the
 * reported point); the polished point replaces the reported one when it is primal and dual
 * feasible within 1e-9, and items (may be NULL) receive the new status, objective and
 * residuals. info[k].status: 0 polished, 1 degenerate optimum, 2 CG not converged, 4 LP not
 * converged, 5 polished point rejected. */
SGB_API int sankhya_gb300_batch_polish(sankhya_gb300_batch* batch,
                                       sankhya_gb300_batch_item* items,
                                       sankhya_gb300_adjoint_info* info);

SGB_API int sankhya_gb300_batch_adjoint(sankhya_gb300_batch* batch,
                                        const double* const* dl_dx, const double* const* dl_dy,
                                        const double* dl_df, double* const* dl_dc,
                                        double* const* dl_drl, double* const* dl_dru,
                                        double* const* dl_dl, double* const* dl_du,
                                        sankhya_gb300_adjoint_info* info);

/* ---- Convex QP --------------------------------------------------------------------------
 * The reference's convex-QP engine on the device: Condat-Vu's primal-dual splitting with a
 * forward step on the quadratic term (src/qp/qp_condat_vu.cpp:164-362), every iterate
 * resident on the GPU. It replaces the body of
 *     Solution sankhya::qp::solve_convex_qp(const Model&, const Options&, Logger&,
 *                                           SolveControl*)          (include/sankhya/qp.hpp:20)
 * behind the seam sankhya::gpu::solve_convex_qp_gpu (sih-26_gb300/seam/qp_gpu.cpp), which runs
 * the reference's own convexity test (src/qp/convexity.cpp:177) before it calls these
 * functions. The engine itself refuses only what it can decide cheaply: a Hessian with a
 * diagonal entry that is negative in minimisation sense (sense * Q_jj below -1e-10 times the
 * largest |Q_jj|, or -1e-10 when that is under 1; the first certificate check_convexity_dense
 * looks for, src/qp/convexity.cpp:89-100) fails to load with SANKHYA_GB300_ERROR_MODEL. A
 * caller that bypasses the seam owns the rest of the convexity decision. */
typedef struct sankhya_gb300_qp sankhya_gb300_qp; /* opaque engine handle */

/* A QP in sankhya::Model's layout: the LP part as sankhya_gb300_lp, and Model::hessian, the
 * stored lower triangle of the symmetric Q as a cols x cols CSC (int32 indices, FP64
 * values), so that the objective is objective_offset + c'x + 0.5 x'Qx and a stored
 * off-diagonal entry (i, j) stands for both Q_ij and Q_ji. hessian_starts may be NULL for no
 * quadratic term. */
typedef struct sankhya_gb300_qp_problem {
  sankhya_gb300_lp lp;
  const int32_t* hessian_starts; /* cols + 1, or NULL */
  const int32_t* hessian_index;
  const double* hessian_values;
} sankhya_gb300_qp_problem;

typedef struct sankhya_gb300_qp_params {
  double tolerance;         /* qp_tolerance: primal and dual residual bound */
  int64_t iteration_limit;  /* iteration_limit; < 0: the engine's ceiling of 1,000,000 */
  double time_limit;        /* seconds; <= 0 is a zero budget, >= 1e300 means none */
  int64_t random_seed;      /* random_seed (both power-iteration starts) */
  int32_t periods_per_poll; /* 50-iteration check periods per CUDA-graph launch; 0 = auto */
  int32_t column_lanes;     /* threads per column in the column pass: 1..32, 0 = auto */
  int32_t row_lanes;        /* threads per row in the row pass: 1..32, 0 = auto */
  int32_t staging;          /* 1: one-lane passes stage each warp's matrix slice in shared
                               memory (the same sums; measured slower on GB300, so 0 is the
                               default) */
  const volatile int32_t* interrupt; /* an interrupt flag, polled; may be NULL */
  sankhya_gb300_log_fn log;  /* every 5,000 iterations, as the reference logs; may be NULL */
  void* log_user;
  sankhya_gb300_poll_fn poll; /* may be NULL */
  void* poll_user;
} sankhya_gb300_qp_params;

typedef struct sankhya_gb300_qp_result {
  int32_t status;  /* OPTIMAL, ITERATION_LIMIT, TIME_LIMIT or INTERRUPTED */
  int32_t ceiling; /* 1 when the iteration limit was the engine's own ceiling */
  int64_t iterations;
  double primal_residual; /* max row-bound violation at the last check; -1 before the first */
  double dual_residual;   /* max |x - proj(x - gradient)| at the last check; -1 before it */
  double norm_a, norm_q;  /* the power-iteration estimates of ||A|| and ||Q|| */
  double tau, sigma;      /* the step sizes */
  double objective;       /* objective_offset + c'x + 0.5 x'Qx at the reported point */
  double setup_seconds;   /* norms and step sizes, on the device */
  double loop_seconds;    /* the iterations */
  double solve_seconds;   /* the whole call, host clock */
  double device_seconds;  /* the whole solve, CUDA events on the engine's stream */
  int64_t kernel_launches; /* engine kernels launched by this solve (graph nodes included) */
  int32_t column_lanes, row_lanes; /* the lanes the passes ran with */
  char message[256];
} sankhya_gb300_qp_result;

SGB_API int sankhya_gb300_qp_create(int32_t device, sankhya_gb300_qp** out);
SGB_API int sankhya_gb300_qp_destroy(sankhya_gb300_qp* engine);
/* Copies the QP to the device: A as CSC and CSR, Q as the full symmetric matrix by rows.
 * Fails with SANKHYA_GB300_ERROR_MODEL on the LP part's defects (as sankhya_gb300_pdhg_load,
 * an infinite cost included), on a Hessian whose structure is not well formed or whose values
 * are not finite, and on a negative diagonal entry as above. */
SGB_API int sankhya_gb300_qp_load(sankhya_gb300_qp* engine,
                                  const sankhya_gb300_qp_problem* problem);
SGB_API int sankhya_gb300_qp_solve(sankhya_gb300_qp* engine,
                                   const sankhya_gb300_qp_params* params,
                                   sankhya_gb300_qp_result* result);
/* The reported point of the last solve, filled as solve_convex_qp fills Solution
 * (src/qp/qp_condat_vu.cpp:343-353): col_value = x, col_dual = c + Qx + sense * A'y,
 * row_dual = -sense * y. Any pointer may be NULL. */
SGB_API int sankhya_gb300_qp_solution(sankhya_gb300_qp* engine, double* col_value,
                                      double* col_dual, double* row_dual);
/* Measurement hook: `reps` iterations on the state the last solve left, each pass bracketed
 * by CUDA events on the engine's stream; ms[0] = mean column pass, ms[1] = mean row pass, in
 * milliseconds. The solve's point is restored afterwards. */
SGB_API int sankhya_gb300_qp_time_kernels(sankhya_gb300_qp* engine, int32_t reps, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* SANKHYA_GB300_H */

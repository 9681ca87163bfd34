// kernels.cuh -- the device control block and the launchers of every engine kernel.
//
// The loop state of the reference's PDHG (src/pdhg/pdhg.cpp:181-197: eta, omega, iteration,
// restarts, the restart KKT, the best residuals) lives in ONE device struct, `Ctl`, which
// the kernels read and the last block of each reducing kernel updates. The host never
// touches it inside the loop; it reads a copy of it (a snapshot) every few steps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "chunks.cuh"
#include "tiles.cuh"

namespace sgb {

// Mirrors sankhya::pdhg::Residuals (src/pdhg/pdhg_evaluate.hpp:19-70).
struct Residuals {
  double primal, dual, gap;
  double primal_objective, dual_objective;
  double absolute_primal, absolute_dual;
  double gap_as_verified, complementarity;
};

__host__ __device__ inline double worst(const Residuals& r) {
  double w = r.primal;
  if (w < r.dual) w = r.dual;
  if (w < r.gap) w = r.gap;
  return w;
}

// src/pdhg/pdhg_evaluate.hpp:57-60; tolerances from include/sankhya/tolerances.hpp:19,22,108.
__host__ __device__ inline bool meets_request(const Residuals& r, double tolerance) {
  return r.primal <= tolerance && r.dual <= tolerance && r.gap <= tolerance &&
         r.absolute_primal <= 1e-7;
}
// src/pdhg/pdhg_evaluate.hpp:65-69.
__host__ __device__ inline bool meets_project_standard(const Residuals& r) {
  return r.absolute_primal <= 1e-7 && r.absolute_dual <= 1e-7 && r.gap_as_verified <= 1e-9 &&
         r.complementarity <= 1e-6;
}

// kRestartRound: the mixed method's inner loop decided a restart, which ends a refinement
// round (the anchor moves to the current iterate and the correction is rescaled).
enum DoneCode : int {
  kRunning = 0, kConverged = 1, kIterationLimit = 2, kFault = 3, kRestartRound = 4
};

constexpr int kLogRing = 64;

// One iteration-table row (Logger::iteration, src/pdhg/pdhg.cpp:399-400).
struct EvalRecord {
  long long iteration;
  double primal_objective;  // minimise space, unscaled
  double primal, dual, gap;
};

// Ticket slots (last-block counters), one per reducing kernel.
enum Ticket : int { kTicketDual = 0, kTicketEvalRows = 1, kTicketPrimal = 2, kTicketEvalCols = 3,
                    kTicketApply = 4, kTicketCount = 5 };

struct Ctl {
  // Step size and primal weight, src/pdhg/pdhg.cpp:181-186.
  double eta, omega, spectral_norm, eta_ceiling, restart_kkt, tolerance;
  long long iteration, averaged, last_restart, restarts, attempts, evaluations;
  long long iteration_limit;
  int cur;          // which of the two x / y buffers holds the current iterate
  int pending_add;  // the last step was accepted and its iterate is not yet in the sums
  int eval_now;     // an evaluation is due: set by the step decision, cleared by the
                    // evaluation's last kernel; steps do nothing while it is set
  int done;         // DoneCode
  int use_restarts, stop_at_request, no_information, accepted;
  int copy_best;    // 0: nothing; 1: the current candidate; 2: the average candidate
  int do_restart;
  int final_mode;   // the evaluation kernels evaluate (best_x, best_y) only
  int stop_rule;    // 0: the reference's stopping test; 1: relative KKT only
  int error;        // a bounded wait gave up (nonzero: the host stops with an error)
  int inner_mode;   // the mixed method's inner loop: a restart ends the round
  double movement, interaction;  // of the last attempted step
  double mv_primal;              // primal half of the movement, from k_primal's last block
  // Mixed method, one refinement round (the FP32 inner loop reads these): the primal and
  // dual scale factors of the correction problem, the scaled problem's bound and cost
  // norms, the scaled objective at the round's anchor, and the round's KKT target.
  double dp, dd, bound_norm_s, cost_norm_s, pobj0, round_target;
  Residuals best;
  Residuals final_residuals;
  double model_objective;  // sum of the original-sense costs times best_x (final mode)
  long long log_count;
  EvalRecord log[kLogRing];
  unsigned int ticket[kTicketCount];
};

constexpr int kEvalColSlots = 16;  // doubles per block in the column-evaluation partials
constexpr int kEvalRowSlots = 8;

struct StepBuffers {
  Ctl* ctl;
  TileSet<double> csc, csr;  // scaled
  double* x[2];
  double* y[2];
  double* x_sum;
  double* y_sum;
  // (2 x' - x, x' - x) of the step, written by k_primal and gathered by k_dual as ONE
  // 16-byte element per entry: a scattered gather costs a cache sector whatever it reads.
  double2* xd;
  const double *c, *l, *u, *rl, *ru;  // scaled problem
  double* part_primal;   // [grid_primal]
  double* part_dual;     // [grid_dual * 2]
  double* chunk_primal;  // [csc.nchunks]
  double* chunk_dual;    // [csr.nchunks * 2]
  int grid_primal, grid_dual;
  int smem_primal, smem_dual;  // dynamic shared memory: pipeline + staged window
  // The step-size factors by iteration count (decisions.cuh, step_factors).
  const double2* step_factors;
  long long step_factors_n;
};

struct EvalBuffers {
  Ctl* ctl;
  TileSet<double> csc, csr;  // UNSCALED values
  const double* x[2];
  const double* y[2];
  double* x_sum;
  double* y_sum;
  double *x_rst, *y_rst;
  const double *dr, *dc;          // row / column scale (Dr, Dc)
  const double* cost;             // minimise-space unscaled cost
  const double* col_cost;         // original-sense cost (for the model objective)
  const double *l, *u, *rl, *ru;  // unscaled bounds
  double bound_norm, cost_norm, sense;
  double *xu[2], *yu[2];  // unscaled candidates (current, average)
  double* reduced;        // reduced cost of candidate 0
  double* best_x;
  double* best_y;
  double* part_rows0;  // [grid_rows * kEvalRowSlots]
  double* part_cols;   // [(grid_cols + 1) * kEvalColSlots]; the last slot holds long columns
  double* part_rows1;  // [grid_rows * kEvalRowSlots]
  double* chunk_cols;  // [csc.nchunks * 2]
  double* chunk_rows;  // [csr.nchunks * 2]
  int grid_rows, grid_cols;
  int m, n;
};

// ---- Launchers (pdhg_kernels.cu) ---------------------------------------------------------
void launch_pdhg_step(const StepBuffers& b, cudaStream_t s);
void launch_primal_pass(const StepBuffers& b, cudaStream_t s);
void launch_dual_pass(const StepBuffers& b, cudaStream_t s);
// Kernels launched per attempted step inside a graph (2 step + 4 evaluation kernels).
// A step graph holds `steps` attempted steps (k_primal + k_dual) and, after every
// kEvalStride of them, the four evaluation kernels. A step that falls due for an evaluation
// sets ctl->eval_now; the steps after it in the graph return at once until the evaluation
// kernels have run and cleared the flag, so the iterates, step sizes and evaluation points
// are those of one evaluation after every due step. The stride divides the 40-step
// evaluation cadence, so on accepted steps the due step ends a stride and nothing is
// skipped. Off a due step the four evaluation kernels return at once.
constexpr int kEvalStride = 8;
inline long long graph_kernel_launches(int steps) {
  return 2LL * steps + 4LL * ((steps + kEvalStride - 1) / kEvalStride);
}
// Running count of kernel launches issued by the launchers of this file (host side).
long long kernel_launch_count();
// The evaluation tick (no-op on the device unless ctl->eval_now or ctl->final_mode).
void launch_evaluation(const EvalBuffers& e, cudaStream_t s);

// Setup kernels.
void launch_scaling_round(int m, int n, TileSet<double> csr, TileSet<double> csc, double* csr_val,
                          double* csc_val, double* row_acc, double* col_acc, double* dr,
                          double* dc, int sum_mode, cudaStream_t s);
void launch_scale_vectors(int m, int n, const double* cost, const double* l, const double* u,
                          const double* rl, const double* ru, const double* dr, const double* dc,
                          double* cs, double* ls, double* us, double* rls, double* rus,
                          cudaStream_t s);
// Fixed device scratch of the allocation-free product: chunk partials for at most
// kNoAllocMaxChunks chunk tiles, its completion counter and its error word. Set up once per
// device (the symbol addresses, and the counter and error word cleared to zero) under a
// lock; later calls only read the cached addresses.
constexpr int kNoAllocMaxChunks = 16384;
cudaError_t noalloc_scratch(int device, cudaStream_t s, double** chunks, unsigned int** ticket,
                            unsigned int** error);

// y = A x with the tile kernel (CSR gives A x; CSC gives A^T x). chunk holds a.nchunks
// doubles; ticket is one device counter that is zero on entry and on exit. A bounded wait
// that gives up sets *error (which the caller clears and reads) and leaves NaN in the rows
// the product could not finish.
// table[e] = step_factors(e) for e < n (decisions.cuh).
void launch_step_factors(double2* table, long long n, cudaStream_t s);
void launch_spmv(TileSet<double> a, const double* x, double* y, double* chunk,
                 unsigned int* ticket, unsigned int* error, cudaStream_t s, int grid);
// out[0] = sum v^2, deterministic; part holds grid doubles.
void launch_sumsq(const double* v, int count, double* part, double* out, unsigned int* ticket,
                  cudaStream_t s, int grid);
void launch_scale_div(double* v, int count, const double* by_sqrt_of, cudaStream_t s);
void launch_abs_minmax(const double* v, int count, double* part, double* out,
                       unsigned int* ticket, cudaStream_t s, int grid);
void launch_project_start(int n, const double* l, const double* u, double* x, cudaStream_t s);
void launch_fill(double* v, int count, double value, cudaStream_t s);

// Resident tile blocks per SM of the step kernels (occupancy query).
int tile_blocks_per_sm();
// The FP64 step passes (pass 0 = column pass, 1 = row pass): the gathered-vector window
// that fits beside their pipeline, their dynamic shared memory for a window of `wmax`
// elements, and how many of their blocks fit one SM with it.
int fp64_window_capacity(int pass);
int fp64_step_smem(int pass, int wmax);
int fp64_step_blocks_per_sm(int pass, int smem);
// Sets the dynamic shared-memory limits of the FP64 kernels on the current device (once per
// device); false if the device refused.
bool configure_tile_kernels();
// Fills dst[k] = src[map[k]] in FP32 (the values of a split layout's part), k < count.
void launch_gather_values(const double* src, const int* map, float* dst, long long count,
                          cudaStream_t s);

}  // namespace sgb

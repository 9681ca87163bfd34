// kernels.cuh -- the device control block and the launchers of every engine kernel.
//
// The loop state of the reference's PDHG (src/pdhg/pdhg.cpp:181-197: eta, omega, iteration,
// restarts, the restart KKT, the best residuals) lives in ONE device struct, `Ctl`, which
// the kernels read and the last block of each reducing kernel updates. The host never
// touches it inside the loop; it reads a copy of it (a snapshot) every few steps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

enum DoneCode : int { kRunning = 0, kConverged = 1, kIterationLimit = 2 };

constexpr int kLogRing = 64;

// One iteration-table row (Logger::iteration, src/pdhg/pdhg.cpp:399-400).
struct EvalRecord {
  long long iteration;
  double primal_objective;  // minimise space, unscaled
  double primal, dual, gap;
};

struct Ctl {
  // Step size and primal weight, src/pdhg/pdhg.cpp:181-186.
  double eta, omega, spectral_norm, eta_ceiling, restart_kkt, tolerance;
  long long iteration, averaged, last_restart, restarts, attempts, evaluations;
  long long iteration_limit;
  int cur;          // which of the two x / y buffers holds the current iterate
  int pending_add;  // the last step was accepted and its iterate is not yet in the sums
  int eval_now;     // the evaluation tick falls after this step
  int done;         // DoneCode
  int use_restarts, stop_at_request, no_information, accepted;
  int copy_best;    // 0: nothing; 1: the current candidate; 2: the average candidate
  int do_restart;
  int final_mode;   // the evaluation kernels evaluate (best_x, best_y) only
  int pad0;
  double movement, interaction;  // of the last attempted step
  Residuals best;
  Residuals final_residuals;
  double model_objective;  // sum of the original-sense costs times best_x (final mode)
  long long log_count;
  EvalRecord log[kLogRing];
  unsigned int ticket[4];  // last-block counters of the reducing kernels
};

// Device arrays of one loaded LP. Index arrays are shared by the scaled and unscaled value
// arrays: scaling never changes the pattern (src/la/scaling.cpp:29-31).
template <typename V>
struct Matrix {
  const int* ptr;      // rows + 1 (CSR) or cols + 1 (CSC)
  const int* idx;      // nnz
  const V* val;        // nnz
  const int2* tiles;   // row (or column) tiles: [begin, end)
  int ntiles;
  int nrows;           // rows of this layout (m for CSR, n for CSC)
};

// Tile capacity: the products of one tile are staged in shared memory.
constexpr int kTileThreads = 256;
constexpr int kTileCap = 2048;

// ---- Launchers (pdhg_kernels.cu) ---------------------------------------------------------
struct StepBuffers {
  Ctl* ctl;
  Matrix<double> csc, csr;      // scaled
  double* x[2];
  double* y[2];
  double* x_sum;
  double* y_sum;
  const double *c, *l, *u, *rl, *ru;  // scaled problem
  double* part_primal;  // [grid]
  double* part_dual;    // [grid * 2]
  int grid_primal, grid_dual;
};

struct EvalBuffers {
  Ctl* ctl;
  Matrix<double> csc, csr;      // UNSCALED values
  const double* x[2];
  const double* y[2];
  const double* x_sum;
  const double* y_sum;
  const double *x_rst, *y_rst;
  const double *dr, *dc;        // row / column scale (Dr, Dc)
  const double *cost;           // minimise-space unscaled cost
  const double *col_cost;       // original-sense cost (for the model objective)
  const double *l, *u, *rl, *ru;  // unscaled bounds
  double bound_norm, cost_norm, sense;
  double *xu[2], *yu[2];        // unscaled candidates (current, average)
  double* reduced;              // reduced cost of candidate 0
  double* best_x;
  double* best_y;
  double* part_rows0;  // [grid_rows * 8]
  double* part_cols;   // [grid_cols * 16]
  double* part_rows1;  // [grid_rows * 8]
  int grid_rows, grid_cols;
  int m, n;
};

// One attempted PDHG step: primal column pass then dual row pass with the step decision.
void launch_pdhg_step(const StepBuffers& b, cudaStream_t s);
// The evaluation tick (no-op on the device unless ctl->eval_now or ctl->final_mode).
void launch_evaluation(const EvalBuffers& e, const StepBuffers& b, cudaStream_t s);

// Setup kernels.
void launch_scaling_round(int m, int n, Matrix<double> csr, Matrix<double> csc, double* csr_val,
                          double* csc_val, double* row_acc, double* col_acc, double* dr,
                          double* dc, int sum_mode, cudaStream_t s);
void launch_scale_vectors(int m, int n, const double* cost, const double* l, const double* u,
                          const double* rl, const double* ru, const double* dr, const double* dc,
                          double* cs, double* ls, double* us, double* rls, double* rus,
                          cudaStream_t s);
// y = A x with the tile kernel (CSR gives A x; CSC gives A^T x).
void launch_spmv(Matrix<double> a, const double* x, double* y, cudaStream_t s, int grid);
// out[0] = sum v^2, deterministic; part holds grid doubles.
void launch_sumsq(const double* v, int count, double* part, double* out, cudaStream_t s,
                  int grid);
void launch_scale_div(double* v, int count, const double* by_sqrt_of, cudaStream_t s);
void launch_abs_minmax(const double* v, int count, double* part, double* out, cudaStream_t s,
                       int grid);
void launch_project_start(int n, const double* l, const double* u, double* x, cudaStream_t s);
void launch_fill(double* v, int count, double value, cudaStream_t s);

int tile_blocks_per_sm();

}  // namespace sgb

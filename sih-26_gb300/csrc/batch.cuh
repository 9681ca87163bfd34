// batch.cuh -- many LPs in one persistent launch.
//
// A batch is a list of LPs, each solved by ONE thread block from start to finish: the block
// takes the next LP from a queue (largest first), runs the reference's restarted PDHG on it
// -- the same steps, step-size rule, evaluations, restarts and stopping tests as the
// single-LP engine (src/pdhg/pdhg.cpp:76-567), written for one block with block-wide
// deterministic reductions -- and takes the next LP when it is done. Every LP keeps its own
// step size, primal weight, restart anchor and counters (its own Ctl), so thousands of LPs of
// uneven sizes and iteration counts share the GPU with no host round trip per iteration.
//
// LPs may share their constraint matrix (branch-and-bound node relaxations differ only in
// their bounds): the matrix is stored, scaled and its norm estimated once, by a first
// persistent launch over the distinct matrices, and the LPs keep only their own vectors.
//
// With precision MIXED each block runs the mixed method of the single-LP engine on its LP: FP32
// PDHG on the correction problem around an FP64 anchor, the anchor moved at every inner
// restart, and the exact FP64 evaluation deciding convergence (mixed.cuh).
//
// An LP whose iterates drift along a dual ray is reported infeasible: at every evaluation
// the change of the dual iterate since the restart anchor, d, is tested as a Farkas
// certificate of the unscaled problem (min over the box of (A^T d)'x minus the support of
// the row box along d must be positive); see batch_farkas in batch_kernels.cu.
#pragma once

#include "kernels.cuh"

namespace sgb {

constexpr int kBatchThreads = 256;     // scaling launches
constexpr int kBatchMaxThreads = 512;  // the largest block a batched solve runs with
constexpr int kAdjThreads = 512;       // adjoint and polish launches
constexpr int kAdjVectors = 9;         // compact per-LP vectors of the square solves
// The square solves gather from two vectors of |B| entries; they sit in shared memory for
// |B| up to this many (2 x 96 KB), else in global memory.
constexpr int kAdjSmemVec = 12288;

// A distinct constraint matrix. Offsets index the packed arrays of BatchBuffers.
struct BatchMatrix {
  int m, n;
  long long cptr;  // offset of its n + 1 column starts (relative to its own entries)
  long long rptr;  // offset of its m + 1 row starts
  long long col;   // offset of its n-vectors (Dc, column scratch, power vector)
  long long row;   // offset of its m-vectors (Dr, row scratch)
  long long nz;    // offset of its entries in the packed index / value arrays
  long long nnz;
  double spectral_norm;  // written by the scaling launch
  double scaled_min_abs, scaled_max_abs;
};

// One LP of the batch.
struct BatchInstance {
  int matrix;
  int m, n;
  long long col;  // offset of its n-vectors
  long long row;  // offset of its m-vectors
  double sense, offset;
  double bound_norm, cost_norm;  // of the unscaled minimise-space problem
};

// What the block leaves for the host, per LP.
struct BatchOutcome {
  int status;     // SANKHYA_GB300_* solve status
  int converged;
  long long iterations, attempts, restarts, evaluations;
  double objective, dual_bound;
  Residuals final_residuals;
  double farkas_value;  // the certificate's normalised value when status is infeasible
  int error;            // nonzero: a device-side inconsistency (reported as an error)
};

struct BatchBuffers {
  int nmatrices, ninstances;
  const BatchMatrix* matrices;
  BatchMatrix* matrices_out;  // spectral norms written by the scaling launch
  const BatchInstance* instances;
  const int* order;           // instance solve order (largest first)
  unsigned int* queue;        // [0] next matrix, [1] next instance (reset by the host)
  // Matrix arrays (offsets from BatchMatrix).
  const int *csc_ptr, *csc_idx, *csr_ptr, *csr_idx;
  const double *csc_raw, *csr_raw;
  double *csc_s, *csr_s;
  double *dr, *dc, *row_acc, *col_acc, *power_v, *power_av;
  // LP arrays (offsets from BatchInstance).
  const double *cost, *col_cost, *l, *u, *rl, *ru;  // unscaled, minimise-space cost
  double *cs, *ls, *us, *rls, *rus;                  // scaled
  double *x0, *x1, *x_sum, *x_rst, *xu0, *xu1, *best_x, *reduced;
  double2* xd;
  double *y0, *y1, *y_sum, *y_rst, *yu0, *yu1, *best_y;
  double* ray;  // the unscaled dual change tested as a Farkas certificate (m per LP)
  BatchOutcome* outcome;
  // Mixed precision (FP32 inner loop on FP64 refinement rounds; see k_batch_solve_mixed).
  float *csc_f, *csr_f;                                   // scaled values in FP32 (per matrix)
  float *u0, *u1, *u_sum, *u_rst, *cf, *lf, *uf, *uc0, *uc1, *u_best;  // n per LP
  float2* ud;                                             // (2u' - u, u' - u), n per LP
  float *v0, *v1, *v_sum, *v_rst, *gu, *gl, *yhat, *vc0, *vc1, *v_best;  // m per LP
  long long* refinements;                                 // rounds per LP
  // Options.
  double tolerance;
  long long iteration_limit;
  int use_restarts, stop_at_request, stop_rule, detect_infeasibility;
  // The schedule: threads that share a row or column in the matrix passes (a power of two,
  // at most 32; the block size is the launch's).
  int lanes;
};

// The adjoint of a solved batch (batch_kernels.cu, k_batch_adjoint): per LP, upstream
// gradients g_x = dL/dx* (n), g_y = dL/dy* (m, y* the row multipliers as reported, dL/db = y*
// for f*) and g_f = dL/df*, and the gradients of L with respect to the cost, the row bounds
// and the column bounds.
struct AdjointOutcome {
  int basic_cols, active_rows;  // |B| and |R|: equal for a nondegenerate optimum
  int iterations[2];            // conjugate-gradient iterations of the two square solves
  double residual[2];           // their final relative residuals ||h - S u|| / ||h||
  int status;  // 0 ok, 1 degenerate (|B| != |R|), 2 not converged
};

struct AdjointBuffers {
  const double *gx, *gy, *gf;                      // upstream (gx, gy per LP slices; gf per LP)
  double *dc, *dl, *du, *drl, *dru;                // results
  double* kw[kAdjVectors];                         // m-sized compact vectors per LP
  int *bcol, *cpos;                                // basic columns; a column's number in B
  int *rrow, *rpos;                                // active rows; a row's number in R
  int *kcp, *krp;                                  // A_RB's CSC / CSR starts (n+1, m+1 per LP)
  int *kci, *kri;                                  // their entries' positions
  double *kcv, *krv;                               // and values
  const long long* knz;                            // per LP: offset of its entries
  signed char *col_state, *row_state;              // active sets
  AdjointOutcome* outcome;
  int max_iterations;                              // per conjugate-gradient run
  double cg_tolerance;
  int smem_vec;                                    // |B| up to which the gathers use smem
};

void launch_batch_scaling(const BatchBuffers& b, int grid, cudaStream_t s);
// The adjoint and polish launches run kAdjThreads-thread blocks with 2 * a.smem_vec
// doubles of dynamic shared memory; adjoint_blocks_per_sm is their occupancy.
void launch_batch_adjoint(const BatchBuffers& b, const AdjointBuffers& a, int grid,
                          cudaStream_t s);
void launch_batch_polish(const BatchBuffers& b, const AdjointBuffers& a, int grid,
                         cudaStream_t s);
int adjoint_blocks_per_sm(int smem_vec);
// The solve launches run blocks of `threads` threads (a multiple of 32, at most
// kBatchMaxThreads); the occupancy queries are for that block size.
void launch_batch_solve(const BatchBuffers& b, int grid, int threads, cudaStream_t s);
void launch_batch_solve_mixed(const BatchBuffers& b, int grid, int threads, cudaStream_t s);
int batch_mixed_blocks_per_sm(int threads);
int batch_blocks_per_sm(int threads = kBatchThreads);

}  // namespace sgb

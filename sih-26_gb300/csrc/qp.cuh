// qp.cuh -- device layout and kernels of the convex-QP engine (Condat-Vu).
//
// The reference's engine (src/qp/qp_condat_vu.cpp:236-335) iterates
//     x'   = proj_box(x - tau (sense c + sense Q x + A'y))
//     xbar = 2 x' - x
//     y'   = v - sigma proj_C(v / sigma),   v = y + sigma A xbar
// and every 50 iterations measures the worst row violation of A x and the worst
// |x - proj_box(x - gradient)|, stopping when both are within qp_tolerance.
//
// Here one iteration is two kernels:
//   column pass  for each column j: (Qx)_j over row j of the full symmetric Q and (A'y)_j over
//                column j of A, then the projected step and the extrapolation (x' to the
//                other buffer of a pair, xbar);
//   row pass     for each row i: (A xbar)_i over row i of A, then the dual prox in place.
// The check after every 50th iteration is the same two passes in their check form (the row
// pass on A x, the column pass on the gradient at x) plus one single-block kernel that takes
// the decision on the device. A row or column is summed by a group of G lanes (G = 1..32,
// from the mean entries per item); one longer than 64 G entries is cut into chunks of
// kQpChunk entries, each summed by a warp, and the last chunk to finish (a ticket per item)
// adds the chunks' sums in chunk order and runs the item's epilogue. Every sum is taken in a
// fixed order, so a solve is reproducible bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "qp_layout.hpp"

namespace sgb {

constexpr int kQpThreads = 256;
constexpr int kQpWarps = kQpThreads / 32;
// On request (sankhya_gb300_qp_params::staging), one-lane passes stage each warp's slice of the
// matrix (its 32 items' entries, contiguous) in shared memory with coalesced loads, then every
// lane walks its own item there: at most kQpStage entries per warp (a warp whose slice is
// longer reads its items directly). Measured on GB300 it is slower, not faster: the 72 KB a
// block needs halves the resident warps (35% active against 66%), and the copy phase no longer
// overlaps the gathers (1M x 2M QP: column pass 250 against 135 us, row pass 230 against
// 141 us). It stays as an option, with the same sums in the same order.
constexpr int kQpStage = 768;
constexpr int kQpStageBytes = kQpWarps * kQpStage * 12;
constexpr int kQpCheckEvery = 50;   // src/qp/qp_condat_vu.cpp:279
constexpr int kQpMaxPeriods = 64;   // check periods per CUDA graph at most

// Modes of the two passes.
enum QpMode { kQpStep = 0, kQpCheck = 1, kQpReport = 2 };

// Decision state, on the device.
struct QpCtl {
  int done;   // the stopping test held
  int error;  // unused by the kernels, cleared at load
  double tau, sigma, tolerance;  // the solve's step sizes and stopping tolerance
  double inv_sigma;              // RN(1 / sigma), for the row pass's division
  long long base;        // iterations completed before the running graph
  long long limit;       // iteration limit in force (the ceiling when none was set)
  long long iterations;  // iteration at which the test held
  unsigned long long primal_bits, dual_bits;  // running maxima of the running check
  double primal, dual, objective;  // the last check's residuals and objective
  long long checked;               // iteration of the last check (0: none)
};

struct QpHist {
  long long iteration;
  double primal, dual, objective;
};

// Everything the kernels read, by value.
struct QpDev {
  int m, n;
  int col_lanes, row_lanes;
  int stage;  // one-lane passes stage the warp's matrix slice in shared memory
  double sense, offset;
  // A by columns (CSC) and by rows (CSR); Q as the full symmetric matrix by rows.
  const int* a_cs;
  const int* a_ri;
  const double* a_cv;
  const int* a_rs;
  const int* a_ci;
  const double* a_rv;
  const int* q_rs;
  const int* q_ci;
  const double* q_v;  // sense Q
  const double* cost;       // sense c
  const double* col_lower;  // bounds with absent sides as -inf / +inf
  const double* col_upper;
  const double* row_lower;
  const double* row_upper;
  double* x0;   // the iterate pair: iteration t reads buffer t % 2 and writes the other
  double* x1;
  double* xbar;
  double* y;
  double* col_dual;  // report form only
  // Long items.
  const QpChunk* col_chunks;
  int ncol_chunks;
  const QpChunk* row_chunks;
  int nrow_chunks;
  double2* chunk_part;       // per chunk: (Qx, A'y) partials of columns, (A v, -) of rows
  double2* row_chunk_part;
  unsigned int* col_tickets;
  unsigned int* row_tickets;
  double* long_col_obj;      // objective terms of the long columns, by slot
  int nlong_cols;
  // Check partials.
  double* obj_part;          // per short-path block of the column pass
  int col_short_blocks, row_short_blocks;
  QpHist* hist;
};

// Launchers. `k` is the iteration's index inside its graph (0-based), `src` the buffer that
// holds x. Step and check kernels return at once when ctl->done is set or their iteration
// is past ctl->limit.
void qp_launch_column_pass(const QpDev& d, QpCtl* ctl, int mode, int k, int src,
                           cudaStream_t s);
void qp_launch_row_pass(const QpDev& d, QpCtl* ctl, int mode, int k, int src, cudaStream_t s);
// The decision after the check whose last iteration is graph index k (period p).
void qp_launch_decide(const QpDev& d, QpCtl* ctl, int k, int p, cudaStream_t s);
// base += iterations of the graph (capped at the limit) unless done.
void qp_launch_advance(QpCtl* ctl, int graph_iterations, cudaStream_t s);

// Setup: out = M v over the rows of a CSR (`lanes` threads per row, 1..32); sum of a[i] * b[i]
// into *out in a fixed order (partials of kQpDotBlocks blocks, then one block);
// v /= sqrt(*norm2).
constexpr int kQpDotBlocks = 304;
void qp_launch_spmv(int rows, const int* starts, const int* index, const double* values,
                    const double* v, double* out, int lanes, cudaStream_t s);
void qp_launch_dot(const double* a, const double* b, int n, double* partials, double* out,
                   cudaStream_t s);
void qp_launch_scale(double* v, int n, const double* norm2, cudaStream_t s);
// row_dual = -sense * y.
void qp_launch_row_dual(const QpDev& d, double* row_dual, cudaStream_t s);
// x0 = proj_box(0) (src/qp/qp_condat_vu.cpp:213-217), y = 0.
void qp_launch_init(const QpDev& d, cudaStream_t s);
long long qp_kernel_launch_count();
// Opts the staged one-lane passes into kQpStageBytes of dynamic shared memory on the current
// device; returns the CUDA error of the first attribute call that failed.
cudaError_t qp_configure_kernels();

}  // namespace sgb

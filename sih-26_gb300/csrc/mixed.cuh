// mixed.cuh -- the mixed-precision method: FP32 PDHG on FP64 refinement rounds.
//
// Round k holds an FP64 anchor (xbar, ybar) of the scaled problem and solves, in FP32, the
// CORRECTION problem in u = Dp (x - xbar), v = Dd (y - ybar):
//     min_u max_v  cf'u + v'A u - Psi(v),   u in [lf, uf],
//     cf = Dd (c + A'ybar),  lf = Dp (l - xbar),  uf = Dp (u - xbar),
// where Psi is the support function of the row box shifted to the anchor. Its proximal step
// is the reference's Moreau step written in correction form with gu = Dp (A xbar - ru),
// gl = Dp (A xbar - rl) and yhat = Dd ybar:
//     t = (yhat + v) / sigma + A ubar
//     v' = v + sigma (gu + A ubar)   if t + gu > 0        (upper side binds)
//     v' = v + sigma (gl + A ubar)   if t + gl < 0        (lower side binds)
//     v' = -yhat                     otherwise            (multiplier leaves the row)
// and on an equality row (gu == gl) simply v' = v + sigma (gu + A ubar). The scale factors
// Dp, Dd are the inverse primal and dual residuals of the anchor, so the correction data are
// O(1) and FP32 resolves them to its own relative precision; each round therefore gains
// several digits on the FP64 point xbar + u / Dp, ybar + v / Dd (iterative refinement for
// LP, Gleixner, Steffy & Wolter, INFORMS J. Computing 28(3), 2016, applied to the saddle
// form). The inner loop's step size, primal weight and KKT norms are FP64; its restart and
// round-end tests use the scaled problem's KKT estimated in correction form; every round ends
// with the exact FP64 evaluation of the reference (src/pdhg/pdhg_evaluate.cpp) on the
// unscaled problem, which alone decides convergence.
#pragma once

#include "kernels.cuh"
#include "tiles.cuh"

namespace sgb {

struct MixedBuffers {
  Ctl* ctl;                  // the inner loop's control block
  TileSet<float> csc, csr;   // scaled values in FP32 (evaluation tile layouts)
  ChunkSet<float> csc_k, csr_k;  // the step passes' chunk layouts
  float* u[2];
  float* v[2];
  float* u_sum;
  float* v_sum;
  float* u_rst;
  float* v_rst;
  float* du;                   // u' - u per column, gathered by the row pass
  // A u of the iterate, double-buffered with u. The row pass gathers only du and forms
  // A ubar = A u + 2 A du and A u' = A u + A du. The rounding that the carried sum picks up
  // cannot build up: every evaluation (at most 40 accepted steps apart) stores A u computed
  // afresh from u, and u = 0, so A u = 0, at the start of every round.
  float* au[2];
  const float *cf, *lf, *uf;   // correction cost and box (n)
  const float* cs;             // scaled cost c-hat (n): the objective of the correction
  const float *gu, *gl, *yhat; // correction row data (m)
  float* uc[2];                // evaluation candidates: current, average
  float* vc[2];
  float* u_best;
  float* v_best;
  double* part_primal;   // [grid_primal]
  double* part_dual;     // [grid_dual * 2]
  double* piece_primal;  // [csc_k.npieces]
  double* piece_dual;    // [csr_k.npieces]
  double* part_rows0;    // [grid_dual * kEvalRowSlots]
  double* part_cols;     // [(grid_primal + 1) * kEvalColSlots]
  double* part_rows1;    // [grid_dual * kEvalRowSlots]
  double* chunk_cols;    // [csc.nchunks * 2]
  double* chunk_rows;    // [csr.nchunks * 2]
  int grid_primal, grid_dual;     // evaluation passes
  int grid_step_primal, grid_step_dual;  // step passes (one block of kChunkThreads per SM)
  int smem_primal, smem_dual;     // step passes' dynamic shared memory
  int m, n;
  const double2* step_factors;    // the step-size factors by iteration count
  long long step_factors_n;
};

// FP64 buffers of the refinement rounds.
struct RoundBuffers {
  Ctl* ctl;              // the inner loop's control block (dp, dd, pobj0 are written here)
  int m, n;
  const double *cs, *ls, *us, *rls, *rus;  // scaled problem (absent bounds = +-inf)
  const double *dr, *dc;
  double *xbar, *ybar;   // the anchor
  double *ax, *aty;      // A xbar, A^T ybar (scaled, FP64)
  float *cf, *lf, *uf, *gu, *gl, *yhat;
  const float *u_src, *v_src;  // the correction the anchor moves by (host-chosen per round)
  double* best_x;        // unscaled (x, y) for the exact FP64 evaluation
  double* best_y;
  double* part;          // [2 * grid] measure partials
  double* out;           // [4]: primal residual (inf-norm), dual residual (inf-norm), c'xbar
  unsigned int* ticket;
  int grid;
};

void launch_mixed_step(const MixedBuffers& b, cudaStream_t s);
void launch_mixed_primal(const MixedBuffers& b, cudaStream_t s);
void launch_mixed_dual(const MixedBuffers& b, cudaStream_t s);
void launch_mixed_evaluation(const MixedBuffers& b, cudaStream_t s);
// Residual measures of the anchor (needs ax, aty computed): out[0..2].
void launch_round_measure(const RoundBuffers& r, cudaStream_t s);
// The correction problem of the round from the anchor and ctl->dp, ctl->dd (host-set).
void launch_round_build(const RoundBuffers& r, cudaStream_t s);
// xbar += u_best / dp (clamped to the box), ybar += v_best / dd; best_x = xbar Dc,
// best_y = ybar Dr for the exact evaluation.
void launch_round_update(const RoundBuffers& r, cudaStream_t s);
void launch_to_float(const double* src, float* dst, long long count, cudaStream_t s);
void launch_fill_float(float* v, int count, float value, cudaStream_t s);
// Sets the dynamic shared-memory limits of the FP32 kernels on the current device (once per
// device); false if the device refused.
bool configure_mixed_kernels();
// Resident FP32 evaluation tile blocks per SM (occupancy query).
int mixed_blocks_per_sm();
// The FP32 step passes (pass 0 = column pass, 1 = row pass): window capacity and dynamic
// shared memory for a window of `wmax` elements (one block of kChunkThreads per SM).
int mixed_window_capacity(int pass);
int mixed_step_smem(int pass, int wmax);

}  // namespace sgb

// mixed_kernels.cu -- the FP32 inner loop and the FP64 refinement rounds (see mixed.cuh).
//
// The step kernels mirror k_primal / k_dual with FP32 values, iterates and FP32-accumulated
// products; the movement and interaction partials are promoted to FP64 at the block level,
// and the step-size decision, restarts and primal weight (decisions.cuh) are FP64. The column
// pass writes du = u' - u per column; the row pass gathers only du (4 bytes per nonzero,
// measured markedly faster on GB300 than an 8-byte (ubar, du) gather) and forms
// A ubar = A u + 2 A du with A u carried per row (MixedBuffers::au). A du comes straight
// from the gather, so the interaction term of the step-size rule keeps FP32's relative
// accuracy however small the step is, rather than being the difference of two large
// products. (On the 1M x 2M block-angular LP both forms took the same number of iterations
// to relative KKT 1e-8.)
#include "common.cuh"
#include "decisions.cuh"
#include "kernels.cuh"
#include "mixed.cuh"
#include "tiles.cuh"

#include <algorithm>
#include <mutex>

namespace sgb {

namespace {

constexpr int kScratch = 16 * (kWideBlockThreads / 32);
constexpr int kChunkScratch = 2 * (kChunkThreads / 32);
// The FP32 evaluation tile blocks run 16 consumer warps (the FP32 layouts' lanes are chosen
// for them).
using EvalPipeF = TilePipe<float, 2, 0, kWideThreads>;
constexpr int kSmemF = EvalPipeF::bytes();
// The step passes' chunk geometry: 256 entries per chunk, one gathered float per entry (v in
// the column pass, du in the row pass).
using StepSmemF = ChunkSmem<float, float, 1, kChunkCapF>;

// A value formed by thread 0 and handed to every thread of the block (all threads call it).
template <typename F>
__device__ __forceinline__ float block_scalar(F f) {
  __shared__ float s_value;
  if (threadIdx.x == 0) s_value = f();
  __syncthreads();
  return s_value;
}

__device__ __forceinline__ void raise_error(Ctl* c) {
  c->error = 1;
  c->done = kFault;
}

__device__ __forceinline__ int grid_stride_begin() {
  return blockIdx.x * blockDim.x + threadIdx.x;
}

// ---- Inner step ----------------------------------------------------------------------------
__global__ void __launch_bounds__(kChunkThreads, 1) k_primal_f(MixedBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kChunkScratch];
  grid_dependency_wait();  // the previous kernel's results (launch_after)
  Ctl* ctl = b.ctl;
  // Every control field the pass reads, loaded together before the first test.
  const int done = ctl->done, eval_now = ctl->eval_now, cur = ctl->cur;
  const bool add = ctl->pending_add != 0;
  const long long iteration = ctl->iteration, limit = ctl->iteration_limit;
  const double omega = ctl->omega, eta = ctl->eta;
  if (done != kRunning || eval_now != 0) return;
  if (iteration >= limit) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->done = kIterationLimit;
    return;
  }
  const float* __restrict__ u = b.u[cur];
  float* __restrict__ un = b.u[cur ^ 1];
  const float* __restrict__ v = b.v[cur];
  // The step's FP32 scalar, formed once per block: GB300 runs FP64 at 1/64 of the FP32 rate,
  // so an FP64 division in each of 1,024 threads would hold the FP64 pipe for thousands of
  // cycles per SM at the start of every launch.
  const float tau = block_scalar([&] { return static_cast<float>(eta / omega); });
  float mvf = 0.0f;
  // Operands of column j: u, cf, lf, uf and (when the last step is still to be added) u_sum.
  auto load = [&](int j, float* o) {
    o[0] = u[j];
    o[1] = b.cf[j];
    o[2] = b.lf[j];
    o[3] = b.uf[j];
    o[4] = add ? b.u_sum[j] : 0.0f;
  };
  auto epi = [&](int j, const float* s, const float* o) {
    const float uj = o[0];
    if (add) b.u_sum[j] = o[4] + uj;
    const float g = o[1] + s[0];
    const float unj = clamp_box(fmaf(-tau, g, uj), o[2], o[3]);
    un[j] = unj;
    const float d = unj - uj;
    b.du[j] = d;
    mvf = fmaf(d, d, mvf);
  };
  if (!run_chunks<1, 5, float, float, kChunkCapF>(b.csc_k, v, dsmem, b.piece_primal, load,
                                                  epi) &&
      threadIdx.x == 0) {
    raise_error(ctl);
  }
  double mv[1] = {static_cast<double>(mvf)};
  if (b.csc_k.nlong == 0) {
    // No long column to finish: each block publishes its partial, and the row pass's last
    // block sums them in block order (primal_movement) when it takes the step decision. No
    // block of this pass waits for another.
    double out[1];
    block_sum<1>(mv, scratch, out);
    if (threadIdx.x == 0) b.part_primal[blockIdx.x] = out[0];
    return;
  }
  if (!arrive_last<1>(mv, scratch, b.part_primal, &ctl->ticket[kTicketPrimal])) return;
  mvf = 0.0f;
  run_chunk_long_rows<1, 5, float>(b.csc_k, b.piece_primal, load, epi);
  mv[0] = static_cast<double>(mvf);
  double longs[1], total[1];
  block_sum<1>(mv, scratch, longs);
  sum_partials<1>(b.part_primal, gridDim.x, scratch, total);
  if (threadIdx.x == 0) {
    ctl->mv_primal = 0.5 * omega * (total[0] + longs[0]);
    ctl->ticket[kTicketPrimal] = 0;
  }
}

__global__ void __launch_bounds__(kChunkThreads, 1) k_dual_f(MixedBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kChunkScratch];
  grid_dependency_wait();  // the previous kernel's results (launch_after)
  Ctl* ctl = b.ctl;
  const int done = ctl->done, eval_now = ctl->eval_now, cur = ctl->cur;
  const bool add = ctl->pending_add != 0;
  const double omega = ctl->omega, eta = ctl->eta;
  if (done != kRunning || eval_now != 0) return;
  // The step-size factors of this step, loaded now for the decision the last block takes.
  const double2 factors = threadIdx.x == 0
                              ? step_factors(ctl->iteration, b.step_factors, b.step_factors_n)
                              : make_double2(0.0, 0.0);
  const float* __restrict__ v = b.v[cur];
  float* __restrict__ vn = b.v[cur ^ 1];
  const float* __restrict__ au = b.au[cur];
  float* __restrict__ aun = b.au[cur ^ 1];
  const float sigma = block_scalar([&] { return static_cast<float>(eta * omega); });
  const float inv_sigma = 1.0f / sigma;
  float a0 = 0.0f, a1 = 0.0f;  // sum dv^2, sum dv (A du)
  // Operands of row i: v, gu, gl, yhat, A u and (when the last step is still to be added)
  // v_sum.
  auto load = [&](int i, float* o) {
    o[0] = v[i];
    o[1] = b.gu[i];
    o[2] = b.gl[i];
    o[3] = b.yhat[i];
    o[4] = au[i];
    o[5] = add ? b.v_sum[i] : 0.0f;
  };
  auto epi = [&](int i, const float* s, const float* o) {
    const float vi = o[0];
    if (add) b.v_sum[i] = o[5] + vi;
    const float gu = o[1], gl = o[2];
    const float adu = s[0];
    aun[i] = o[4] + adu;
    const float abar = fmaf(2.0f, adu, o[4]);  // A ubar
    float vni;
    if (gu == gl) {
      vni = fmaf(sigma, gu + abar, vi);
    } else {
      const float yhat = o[3];
      const float t = fmaf(yhat + vi, inv_sigma, abar);
      if (t + gu > 0.0f) {
        vni = fmaf(sigma, gu + abar, vi);
      } else if (t + gl < 0.0f) {
        vni = fmaf(sigma, gl + abar, vi);
      } else {
        vni = -yhat;
      }
    }
    vn[i] = vni;
    const float d = vni - vi;
    a0 = fmaf(d, d, a0);
    a1 = fmaf(d, adu, a1);
  };
  if (!run_chunks<1, 6, float, float, kChunkCapF>(b.csr_k, b.du, dsmem, b.piece_dual, load,
                                                  epi) &&
      threadIdx.x == 0) {
    raise_error(ctl);
  }
  double acc2[2] = {static_cast<double>(a0), static_cast<double>(a1)};
  if (!arrive_last<2>(acc2, scratch, b.part_dual, &ctl->ticket[kTicketDual])) return;
  a0 = a1 = 0.0f;
  run_chunk_long_rows<1, 6, float>(b.csr_k, b.piece_dual, load, epi);
  acc2[0] = a0;
  acc2[1] = a1;
  double longs[2], total[2];
  block_sum<2>(acc2, scratch, longs);
  sum_partials<2>(b.part_dual, gridDim.x, scratch, total);
  const double mv_primal = primal_movement(b.csc_k.nlong == 0, b.part_primal,
                                           b.grid_step_primal, omega, ctl, scratch);
  if (threadIdx.x == 0) {
    ctl->ticket[kTicketDual] = 0;
    if (ctl->done == kRunning) {
      const double movement = mv_primal + (0.5 * (total[0] + longs[0])) / omega;
      step_decision(ctl, movement, fabs(total[1] + longs[1]), factors);
    }
  }
}

// ---- Inner evaluation (correction form, FP64 accumulation) ---------------------------------
__device__ __forceinline__ bool inner_eval_active(const Ctl* c) {
  return c->eval_now != 0 && c->done == kRunning;
}

// Rows, no matrix: the dual candidates (current, average), the row half of the dual
// violation (a multiplier on a row side that does not exist), |v - v_restart|^2.
__global__ void __launch_bounds__(kTileThreads) k_evalf_rows0(MixedBuffers b) {
  __shared__ double scratch[kScratch];
  const Ctl* c = b.ctl;
  if (!inner_eval_active(c)) return;
  const int cur = c->cur;
  const bool avg = c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const float count = static_cast<float>(c->averaged);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int i = grid_stride_begin(); i < b.m; i += gridDim.x * blockDim.x) {
    const float vcur = b.v[cur][i];
    float cand[2] = {vcur, 0.0f};
    if (avg) cand[1] = (pend ? b.v_sum[i] + vcur : b.v_sum[i]) / count;
    const float gu = b.gu[i], gl = b.gl[i], yh = b.yhat[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !avg) break;
      b.vc[q][i] = cand[q];
      const double yc = static_cast<double>(yh) + static_cast<double>(cand[q]);
      if ((yc > 0.0 && isinf(gu)) || (yc < 0.0 && isinf(gl))) acc[q] += yc * yc;
    }
    const double d = static_cast<double>(vcur) - static_cast<double>(b.v_rst[i]);
    acc[2] += d * d;
  }
  double out[3];
  block_sum<3>(acc, scratch, out);
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) b.part_rows0[blockIdx.x * kEvalRowSlots + q] = out[q];
  }
}

// Columns over the FP32 CSC: d_c = cf + A^T v_c of both candidates, the column dual
// violation, the column half of the gap (sum d (x - bound) in correction units), |u-u_rst|^2.
__global__ void __launch_bounds__(kWideBlockThreads) k_evalf_cols(MixedBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* c = b.ctl;
  if (!inner_eval_active(c)) return;
  const int cur = c->cur;
  const bool avg = c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const float count = static_cast<float>(c->averaged);
  const float* __restrict__ vc0 = b.vc[0];
  const float* __restrict__ vc1 = b.vc[1];
  // dviol0, gapc0, dviol1, gapc1, du^2, c'u0, c'u1
  double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  auto gather = [&](int row, float a, float* s) {
    s[0] = fmaf(a, vc0[row], s[0]);
    if (avg) s[1] = fmaf(a, vc1[row], s[1]);
  };
  auto epi = [&](int j, const float* s) {
    const float ucur = b.u[cur][j];
    float cand[2] = {ucur, 0.0f};
    if (avg) cand[1] = (pend ? b.u_sum[j] + ucur : b.u_sum[j]) / count;
    const float lf = b.lf[j], uf = b.uf[j], cf = b.cf[j];
    const double cj = b.cs[j];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !avg) break;
      b.uc[q][j] = cand[q];
      const double d = static_cast<double>(cf) + static_cast<double>(s[q]);
      const double uq = static_cast<double>(cand[q]);
      if (d > 0.0) {
        if (isinf(lf)) acc[2 * q] += d * d; else acc[2 * q + 1] += d * (uq - lf);
      } else if (d < 0.0) {
        if (isinf(uf)) acc[2 * q] += d * d; else acc[2 * q + 1] += d * (uq - uf);
      }
      acc[5 + q] += cj * uq;
    }
    const double d = static_cast<double>(ucur) - static_cast<double>(b.u_rst[j]);
    acc[4] += d * d;
  };
  EvalPipeF pipe;
  pipe.setup(dsmem);
  if (!run_tiles<2, float>(pipe, b.csc, b.chunk_cols, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(c);
  }
  double out[7];
  block_sum<7>(acc, scratch, out);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    double* p = b.part_cols + blockIdx.x * kEvalColSlots;
    for (int q = 0; q < 7; ++q) p[q] = out[q];
    __threadfence();
    s_last = atomicAdd(&c->ticket[kTicketEvalCols], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int q = 0; q < 7; ++q) acc[q] = 0.0;
  run_long_rows<2, float>(b.csc, b.chunk_cols, epi);
  block_sum<7>(acc, scratch, out);
  if (threadIdx.x == 0) {
    double* p = b.part_cols + b.grid_primal * kEvalColSlots;
    for (int q = 0; q < 7; ++q) p[q] = out[q];
    c->ticket[kTicketEvalCols] = 0;
  }
}

__device__ bool round_stop_test(const Ctl* c, const Residuals& r) {
  return worst(r) <= c->round_target;
}

// Rows over the FP32 CSR: A u_c, the primal violation and the row half of the gap; the last
// block assembles the scaled-problem KKT of xbar + u/dp, ybar + v/dd and decides. A u of the
// current iterate (candidate 0) replaces the step passes' carried A u.
__global__ void __launch_bounds__(kWideBlockThreads) k_evalf_rows1(MixedBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* c = b.ctl;
  if (!inner_eval_active(c)) return;
  const bool avg = c->averaged > 0;
  const float* __restrict__ uc0 = b.uc[0];
  const float* __restrict__ uc1 = b.uc[1];
  float* __restrict__ au = b.au[c->cur];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};  // pviol0, gapr0, pviol1, gapr1
  auto gather = [&](int col, float a, float* s) {
    s[0] = fmaf(a, uc0[col], s[0]);
    if (avg) s[1] = fmaf(a, uc1[col], s[1]);
  };
  auto epi = [&](int i, const float* s) {
    au[i] = s[0];
    const double gu = b.gu[i], gl = b.gl[i], yh = b.yhat[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !avg) break;
      const double a = s[q];
      const double eu = gu + a;     // dp ((A x)_i - ru_i)
      const double el = -(gl + a);  // dp (rl_i - (A x)_i)
      const double viol = dmax(0.0, dmax(eu, el));
      acc[2 * q] += viol * viol;
      const double yc = yh + static_cast<double>(b.vc[q][i]);
      if (yc > 0.0 && !isinf(gu)) acc[2 * q + 1] += yc * eu;
      else if (yc < 0.0 && !isinf(gl)) acc[2 * q + 1] += yc * (gl + a);
    }
  };
  EvalPipeF pipe;
  pipe.setup(dsmem);
  if (!run_tiles<2, float>(pipe, b.csr, b.chunk_rows, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(c);
  }
  double sums[4];
  block_sum<4>(acc, scratch, sums);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    double* p = b.part_rows1 + blockIdx.x * kEvalRowSlots;
    for (int q = 0; q < 4; ++q) p[q] = sums[q];
    __threadfence();
    s_last = atomicAdd(&c->ticket[kTicketEvalRows], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int q = 0; q < 4; ++q) acc[q] = 0.0;
  run_long_rows<2, float>(b.csr, b.chunk_rows, epi);
  double s[14];
  for (int q = 0; q < 4; ++q) s[q] = acc[q];
  for (int q = 4; q < 14; ++q) s[q] = 0.0;
  for (int blk = threadIdx.x; blk < b.grid_dual; blk += blockDim.x) {
    for (int q = 0; q < 4; ++q) s[q] += __ldcg(b.part_rows1 + blk * kEvalRowSlots + q);
    for (int q = 0; q < 3; ++q) s[4 + q] += __ldcg(b.part_rows0 + blk * kEvalRowSlots + q);
  }
  for (int blk = threadIdx.x; blk <= b.grid_primal; blk += blockDim.x) {
    for (int q = 0; q < 7; ++q) s[7 + q] += __ldcg(b.part_cols + blk * kEvalColSlots + q);
  }
  double t[14];
  block_sum<14>(s, scratch, t);
  if (threadIdx.x != 0) return;
  c->ticket[kTicketEvalRows] = 0;
  // t: [0] pviol0 [1] gapr0 [2] pviol1 [3] gapr1 [4] rviol0 [5] rviol1 [6] dv^2
  //    [7] cviol0 [8] gapc0 [9] cviol1 [10] gapc1 [11] du^2 [12] c'u0 [13] c'u1
  const double dp = c->dp, dd = c->dd;
  auto assemble = [&](double pv, double gr, double rv, double cv, double gc, double cu) {
    Residuals r;
    r.absolute_primal = sqrt(pv) / dp;
    r.primal = r.absolute_primal / (1.0 + c->bound_norm_s);
    r.absolute_dual = sqrt(cv + rv) / dd;
    r.dual = r.absolute_dual / (1.0 + c->cost_norm_s);
    // Objective of xbar + u / dp; the gap from the complementarity products, so the
    // large and nearly equal primal and dual objectives are never subtracted.
    const double gap = (gc - gr) / (dp * dd);
    r.primal_objective = c->pobj0 + cu / dp;
    r.dual_objective = r.primal_objective - gap;
    r.gap = fabs(gap) / (1.0 + fabs(r.primal_objective) + fabs(r.dual_objective));
    r.gap_as_verified = fabs(gap) / dmax(1.0, fabs(r.primal_objective));
    r.complementarity = 0.0;
    return r;
  };
  const Residuals cur = assemble(t[0], t[1], t[4], t[7], t[8], t[12]);
  Residuals av;
  if (avg) av = assemble(t[2], t[3], t[5], t[9], t[10], t[13]);
  tick_decisions(c, cur, avg ? &av : nullptr, round_stop_test, t[11], t[6], 1e-10, 1e10);
}

// The vector half of the decisions; the last block to finish clears the evaluation flags.
__global__ void k_evalf_apply(MixedBuffers b) {
  Ctl* c = b.ctl;
  if (c->eval_now == 0) return;
  const int copy = c->copy_best;
  const bool restart = c->do_restart != 0;
  const int cur = c->cur;
  const int total = (copy == 0 && !restart) ? 0 : (b.m > b.n ? b.m : b.n);
  for (int k = grid_stride_begin(); k < total; k += gridDim.x * blockDim.x) {
    if (k < b.n) {
      if (copy) b.u_best[k] = b.uc[copy - 1][k];
      if (restart) {
        b.u_rst[k] = b.u[cur][k];
        b.u_sum[k] = 0.0f;
      }
    }
    if (k < b.m) {
      if (copy) b.v_best[k] = b.vc[copy - 1][k];
      if (restart) {
        b.v_rst[k] = b.v[cur][k];
        b.v_sum[k] = 0.0f;
      }
    }
  }
  clear_evaluation_flags(c);
}

// ---- Refinement rounds (FP64) --------------------------------------------------------------

// Residual measures of the anchor: out[0] = max primal violation, out[1] = max dual
// residual (reduced cost not absorbed by the bound the anchor sits on, or a multiplier on a
// row side the activity does not touch), out[2] = c' xbar.
__global__ void k_round_measure(RoundBuffers r) {
  __shared__ double scratch[3 * (kTileThreads / 32)];
  double mx[2] = {0.0, 0.0};
  double obj[1] = {0.0};
  const int total = r.m > r.n ? r.m : r.n;
  for (int k = grid_stride_begin(); k < total; k += gridDim.x * blockDim.x) {
    if (k < r.m) {
      const double a = r.ax[k], rl = r.rls[k], ru = r.rus[k], y = r.ybar[k];
      mx[0] = dmax(mx[0], dmax(rl - a, a - ru));
      if (rl != ru) {
        if (y > 0.0 && a < ru) mx[1] = dmax(mx[1], y);
        if (y < 0.0 && a > rl) mx[1] = dmax(mx[1], -y);
      }
    }
    if (k < r.n) {
      const double d = r.cs[k] + r.aty[k], x = r.xbar[k], l = r.ls[k], u = r.us[k];
      double res;
      if (l == u) res = 0.0;
      else if (x <= l) res = d < 0.0 ? -d : 0.0;
      else if (x >= u) res = d > 0.0 ? d : 0.0;
      else res = fabs(d);
      mx[1] = dmax(mx[1], res);
      obj[0] = fma(r.cs[k], x, obj[0]);
    }
  }
  double m2[2], o1[1];
  block_max<2>(mx, scratch, m2);
  block_sum<1>(obj, scratch, o1);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    r.part[3 * blockIdx.x] = m2[0];
    r.part[3 * blockIdx.x + 1] = m2[1];
    r.part[3 * blockIdx.x + 2] = o1[0];
    __threadfence();
    s_last = atomicAdd(r.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double a[2] = {0.0, 0.0}, o[1] = {0.0};
  for (int blk = threadIdx.x; blk < gridDim.x; blk += blockDim.x) {
    a[0] = dmax(a[0], __ldcg(r.part + 3 * blk));
    a[1] = dmax(a[1], __ldcg(r.part + 3 * blk + 1));
    o[0] += __ldcg(r.part + 3 * blk + 2);
  }
  block_max<2>(a, scratch, m2);
  block_sum<1>(o, scratch, o1);
  if (threadIdx.x == 0) {
    r.out[0] = m2[0];
    r.out[1] = m2[1];
    r.out[2] = o1[0];
    *r.ticket = 0;
  }
}

__global__ void k_round_build(RoundBuffers r) {
  const double dp = r.ctl->dp, dd = r.ctl->dd;
  const int total = r.m > r.n ? r.m : r.n;
  for (int k = grid_stride_begin(); k < total; k += gridDim.x * blockDim.x) {
    if (k < r.n) {
      const double x = r.xbar[k];
      r.cf[k] = static_cast<float>(dd * (r.cs[k] + r.aty[k]));
      r.lf[k] = static_cast<float>(dp * (r.ls[k] - x));
      r.uf[k] = static_cast<float>(dp * (r.us[k] - x));
    }
    if (k < r.m) {
      const double a = r.ax[k];
      r.gu[k] = static_cast<float>(dp * (a - r.rus[k]));
      r.gl[k] = static_cast<float>(dp * (a - r.rls[k]));
      r.yhat[k] = static_cast<float>(dd * r.ybar[k]);
    }
  }
}

__global__ void k_round_update(RoundBuffers r) {
  const double dp = r.ctl->dp, dd = r.ctl->dd;
  const int total = r.m > r.n ? r.m : r.n;
  for (int k = grid_stride_begin(); k < total; k += gridDim.x * blockDim.x) {
    if (k < r.n) {
      const double x = clamp_box(r.xbar[k] + static_cast<double>(r.u_src[k]) / dp, r.ls[k],
                                 r.us[k]);
      r.xbar[k] = x;
      r.best_x[k] = x * r.dc[k];
    }
    if (k < r.m) {
      const double y = r.ybar[k] + static_cast<double>(r.v_src[k]) / dd;
      r.ybar[k] = y;
      r.best_y[k] = y * r.dr[k];
    }
  }
}

__global__ void k_to_float(const double* src, float* dst, long long count) {
  for (long long k = grid_stride_begin(); k < count; k += static_cast<long long>(gridDim.x) * blockDim.x) {
    dst[k] = static_cast<float>(src[k]);
  }
}

__global__ void k_fill_float(float* v, int count, float value) {
  for (int k = grid_stride_begin(); k < count; k += gridDim.x * blockDim.x) v[k] = value;
}

int egrid(long long count) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sms = 1;
  }
  long long blocks = (count + 255) / 256;
  const long long cap = static_cast<long long>(sms) * 8;
  if (blocks > cap) blocks = cap;
  return blocks < 1 ? 1 : static_cast<int>(blocks);
}

// Per-device state: whether the kernels' shared-memory limits are set on the device, and
// the evaluation kernels' occupancy there.
constexpr int kMaxDevices = 64;
struct MixedConfig {
  bool configured;
  int per_sm;
};
std::mutex g_mixed_mutex;
MixedConfig g_mixed[kMaxDevices];

}  // namespace

bool configure_mixed_kernels() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return false;
  }
  std::lock_guard<std::mutex> lock(g_mixed_mutex);
  MixedConfig& c = g_mixed[dev];
  if (c.configured) return true;
  const cudaError_t errs[] = {
      cudaFuncSetAttribute(k_primal_f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           max_dynamic_smem(reinterpret_cast<const void*>(k_primal_f))),
      cudaFuncSetAttribute(k_dual_f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           max_dynamic_smem(reinterpret_cast<const void*>(k_dual_f))),
      cudaFuncSetAttribute(k_evalf_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemF),
      cudaFuncSetAttribute(k_evalf_rows1, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemF)};
  for (cudaError_t e : errs) {
    if (e != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  }
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_evalf_rows1, kWideBlockThreads,
                                                    kSmemF) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_evalf_cols, kWideBlockThreads,
                                                    kSmemF) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  c.per_sm = std::max(1, std::min(a, b));
  c.configured = true;
  return true;
}

int mixed_blocks_per_sm() {
  if (!configure_mixed_kernels()) return 1;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_mixed_mutex);
  return g_mixed[dev].per_sm > 0 ? g_mixed[dev].per_sm : 1;
}

// The window a block of kChunkThreads stages: what is left beside its warp buffers, at most
// kWindowBytesMax, in gathered floats (a multiple of 1024).
int mixed_window_capacity(int pass) {
  configure_mixed_kernels();
  const void* k = pass == 0 ? reinterpret_cast<const void*>(k_primal_f)
                            : reinterpret_cast<const void*>(k_dual_f);
  const int budget =
      std::min(max_dynamic_smem(k) - StepSmemF::bytes(kChunkThreads / 32, 0), kWindowBytesMax);
  return budget > 0 ? (budget / static_cast<int>(sizeof(float))) & ~1023 : 0;
}

int mixed_step_smem(int pass, int wmax) {
  (void)pass;
  return StepSmemF::bytes(kChunkThreads / 32, wmax);
}

// The two step passes are launched with programmatic stream serialization (launch_after):
// each occupies a whole SM, and its blocks are placed as the previous kernel's leave, so the
// launch and the SM's reconfiguration overlap that kernel's last blocks.
void launch_mixed_primal(const MixedBuffers& b, cudaStream_t s) {
  launch_after(k_primal_f, b.grid_step_primal, kChunkThreads, b.smem_primal, s, b);
}

void launch_mixed_dual(const MixedBuffers& b, cudaStream_t s) {
  launch_after(k_dual_f, b.grid_step_dual, kChunkThreads, b.smem_dual, s, b);
}

void launch_mixed_step(const MixedBuffers& b, cudaStream_t s) {
  launch_mixed_primal(b, s);
  launch_mixed_dual(b, s);
}

void launch_mixed_evaluation(const MixedBuffers& b, cudaStream_t s) {
  k_evalf_rows0<<<b.grid_dual, kTileThreads, 0, s>>>(b);
  k_evalf_cols<<<b.grid_primal, kWideBlockThreads, kSmemF, s>>>(b);
  k_evalf_rows1<<<b.grid_dual, kWideBlockThreads, kSmemF, s>>>(b);
  k_evalf_apply<<<egrid(b.m > b.n ? b.m : b.n), 256, 0, s>>>(b);
}

void launch_round_measure(const RoundBuffers& r, cudaStream_t s) {
  k_round_measure<<<r.grid, kTileThreads, 0, s>>>(r);
}

void launch_round_build(const RoundBuffers& r, cudaStream_t s) {
  k_round_build<<<egrid(r.m > r.n ? r.m : r.n), 256, 0, s>>>(r);
}

void launch_round_update(const RoundBuffers& r, cudaStream_t s) {
  k_round_update<<<egrid(r.m > r.n ? r.m : r.n), 256, 0, s>>>(r);
}

void launch_to_float(const double* src, float* dst, long long count, cudaStream_t s) {
  if (count <= 0) return;
  k_to_float<<<egrid(count), 256, 0, s>>>(src, dst, count);
}

void launch_fill_float(float* v, int count, float value, cudaStream_t s) {
  if (count <= 0) return;
  k_fill_float<<<egrid(count), 256, 0, s>>>(v, count, value);
}

}  // namespace sgb

// pdhg_kernels.cu -- the FP64 hot path of the GB300 PDHG engine.
//
// Per attempted step (src/pdhg/pdhg.cpp:220-335) there are TWO kernels, both on the tile
// engine of tiles.cuh (the FP32 method's step kernels run on the warp chunks of chunks.cuh
// instead; on GB300's FP64 pipe these tile kernels measured faster than chunk versions):
//   k_primal  one pass over the CSC copy of Ahat: A^T y gathered per column, fused with the
//             projected primal update x' = proj(x - tau (c + A^T y)), xbar = 2x' - x and
//             dx = x' - x (written once per column so the row pass needs one FMA per entry
//             and product), the primal half of the movement, and the deferred x_sum update.
//   k_dual    one pass over the CSR copy: A xbar and A dx from ONE read of each row, fused
//             with the Moreau dual update, the dual movement and the interaction dy^T A dx;
//             its last block sums every block's partials in a fixed order and takes the
//             step-size decision on the device.
// The evaluation tick (src/pdhg/pdhg.cpp:341-483, src/pdhg/pdhg_evaluate.cpp) is three
// fused passes over the UNSCALED values plus one vector pass; it runs only when the step
// decision asks for it and otherwise returns at once.
//
// GB300 executes FP64 at about 1/64 of its FP32 rate, so this method is bound by the FP64
// pipe rather than by HBM: the kernels are written to spend as few FP64 instructions per
// entry as the method allows (one FMA per entry and product), to divide only where a row
// is not an equality, and to keep every reduction deterministic.
#include "common.cuh"
#include "decisions.cuh"
#include "kernels.cuh"
#include "tiles.cuh"

#include <algorithm>
#include <cstdio>
#include <mutex>

namespace sgb {

namespace {

long long g_launches = 0;

constexpr int kScratch = 16 * (kBlockThreads / 32);
// The step passes keep one tile in flight beside the staged window (a larger window pays
// more in FP64 than a deeper pipeline); each tile brings its
// rows' operands: x, c, l, u, x_sum (column pass) and y, rl, ru, y_sum (row pass).
constexpr int kStepStages = 2;
using PrimalPipe = TilePipe<double, kStepStages, 5>;
using DualPipe = TilePipe<double, kStepStages, 4>;

// Per-device state: whether the kernels' shared-memory limits are set on the device, and
// its occupancy and SM count (an engine on device 1 needs its own opt-in).
constexpr int kMaxDevices = 64;
struct DeviceConfig {
  bool configured;
  int tile_blocks_per_sm;
  int sms;
};
std::mutex g_config_mutex;
DeviceConfig g_config[kMaxDevices];

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return dev >= 0 && dev < kMaxDevices ? dev : -1;
}

int device_sms() {
  const int dev = current_device();
  if (dev < 0) return 1;
  std::lock_guard<std::mutex> lock(g_config_mutex);
  if (g_config[dev].sms == 0) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      sms = 1;
    }
    g_config[dev].sms = sms > 0 ? sms : 1;
  }
  return g_config[dev].sms;
}

__device__ __forceinline__ void raise_error(Ctl* c) {
  c->error = 1;
  c->done = kFault;
}

// The reference's stopping test (src/pdhg/pdhg.cpp:424-425), or relative KKT alone.
__device__ bool fp64_stop_test(const Ctl* c, const Residuals& r) {
  return c->stop_rule == 1 ? worst(r) <= c->tolerance
                           : meets_request(r, c->tolerance) &&
                                 (c->stop_at_request || meets_project_standard(r));
}

// ---- k_primal ----------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlockThreads) k_primal(StepBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* ctl = b.ctl;
  if (ctl->done != kRunning || ctl->eval_now != 0) return;
  if (ctl->iteration >= ctl->iteration_limit) {  // src/pdhg/pdhg.cpp:206
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->done = kIterationLimit;
    return;
  }
  const int cur = ctl->cur;
  const double* x = b.x[cur];
  double* __restrict__ xn = b.x[cur ^ 1];
  const double* __restrict__ y = b.y[cur];
  const double omega = ctl->omega;
  // Formed once per block: an FP64 division per thread would hold GB300's slow FP64 pipe.
  __shared__ double s_tau;
  if (threadIdx.x == 0) s_tau = ctl->eta / omega;
  __syncthreads();
  const double tau = s_tau;
  const bool add = ctl->pending_add != 0;
  double mv[1] = {0.0};  // sum of dx^2
  PrimalPipe pipe;
  pipe.setup(dsmem);
  pipe.rsrc[0] = x;
  pipe.rsrc[1] = b.c;
  pipe.rsrc[2] = b.l;
  pipe.rsrc[3] = b.u;
  pipe.rsrc[4] = b.x_sum;
  Window<double> win;
  win.setup(y, pipe, dsmem);
  auto gather = [&](int row, double v, double* acc) { acc[0] = fma(v, win.get(row), acc[0]); };
  auto epi = [&](int j, const double* s) {
    const double xj = pipe.row(0, j);
    if (add) b.x_sum[j] = pipe.row(4, j) + xj;
    const double gradient = pipe.row(1, j) + s[0];
    // Unfused, as src/pdhg/pdhg.cpp:232-233 rounds it.
    const double xnj =
        clamp_box(__dsub_rn(xj, __dmul_rn(tau, gradient)), pipe.row(2, j), pipe.row(3, j));
    xn[j] = xnj;
    const double d = xnj - xj;
    // 2 x' is exact, so the FMA rounds once, as the reference's 2.0 * x' - x does.
    b.xd[j] = make_double2(fma(2.0, xnj, -xj), d);
    mv[0] = fma(d, d, mv[0]);
  };
  if (!run_tiles<1, double>(pipe, b.csc, win, b.chunk_primal, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(ctl);
  }
  if (b.csc.nlong == 0) {
    // No long column to finish: each block publishes its partial, and k_dual's last block
    // sums them in block order (primal_movement). No block of this pass waits for another.
    double out[1];
    block_sum<1>(mv, scratch, out);
    if (threadIdx.x == 0) b.part_primal[blockIdx.x] = out[0];
    return;
  }
  if (!arrive_last<1>(mv, scratch, b.part_primal, &ctl->ticket[kTicketPrimal])) return;
  mv[0] = 0.0;
  run_long_rows<1>(b.csc, b.chunk_primal, epi);
  double longs[1], total[1];
  block_sum<1>(mv, scratch, longs);
  sum_partials<1>(b.part_primal, gridDim.x, scratch, total);
  if (threadIdx.x == 0) {
    ctl->mv_primal = 0.5 * omega * (total[0] + longs[0]);
    ctl->ticket[kTicketPrimal] = 0;
  }
}

// ---- k_dual ------------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlockThreads) k_dual(StepBuffers b) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* ctl = b.ctl;
  if (ctl->done != kRunning || ctl->eval_now != 0) return;
  const int cur = ctl->cur;
  // The step-size factors of this step, loaded now for the decision the last block takes.
  const double2 factors = threadIdx.x == 0
                              ? step_factors(ctl->iteration, b.step_factors, b.step_factors_n)
                              : make_double2(0.0, 0.0);
  const double* __restrict__ y = b.y[cur];
  double* __restrict__ yn = b.y[cur ^ 1];
  const double2* __restrict__ xd = b.xd;
  const double omega = ctl->omega;
  const double sigma = ctl->eta * omega;
  const bool add = ctl->pending_add != 0;
  double acc2[2] = {0.0, 0.0};  // sum dy^2, sum dy (A dx)
  DualPipe pipe;
  pipe.setup(dsmem);
  pipe.rsrc[0] = y;
  pipe.rsrc[1] = b.rl;
  pipe.rsrc[2] = b.ru;
  pipe.rsrc[3] = b.y_sum;
  Window<double2> win;
  win.setup(xd, pipe, dsmem);
  auto gather = [&](int col, double v, double* acc) {
    const double2 p = win.get(col);
    acc[0] = fma(v, p.x, acc[0]);
    acc[1] = fma(v, p.y, acc[1]);
  };
  auto epi = [&](int i, const double* s) {
    const double yi = pipe.row(0, i);
    if (add) b.y_sum[i] = pipe.row(3, i) + yi;
    const double rl = pipe.row(1, i), ru = pipe.row(2, i);
    // Unfused, as the reference rounds it (src/pdhg/pdhg.cpp:244-245): a fused
    // v - sigma * (v / sigma) would leave the division's rounding error on a free row. On
    // an equality row the projection is the bound whatever v is, so no division is needed.
    const double v = __dadd_rn(yi, __dmul_rn(sigma, s[0]));
    const double p = rl == ru ? rl : clamp_box(v / sigma, rl, ru);
    const double yni = __dsub_rn(v, __dmul_rn(sigma, p));
    yn[i] = yni;
    const double d = yni - yi;
    acc2[0] = fma(d, d, acc2[0]);
    acc2[1] = fma(d, s[1], acc2[1]);
  };
  if (!run_tiles<2, double>(pipe, b.csr, win, b.chunk_dual, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(ctl);
  }
  if (!arrive_last<2>(acc2, scratch, b.part_dual, &ctl->ticket[kTicketDual])) return;
  acc2[0] = acc2[1] = 0.0;
  run_long_rows<2>(b.csr, b.chunk_dual, epi);
  double longs[2], total[2];
  block_sum<2>(acc2, scratch, longs);
  sum_partials<2>(b.part_dual, gridDim.x, scratch, total);
  const double mv_primal =
      primal_movement(b.csc.nlong == 0, b.part_primal, b.grid_primal, omega, ctl, scratch);
  if (threadIdx.x == 0) {
    ctl->ticket[kTicketDual] = 0;
    if (ctl->done == kRunning) {
      const double movement = mv_primal + (0.5 * (total[0] + longs[0])) / omega;
      step_decision(ctl, movement, fabs(total[1] + longs[1]), factors);
    }
  }
}

// ---- Evaluation ----------------------------------------------------------------------------
__device__ __forceinline__ bool eval_active(const Ctl* c) {
  return c->final_mode != 0 || (c->eval_now != 0 && c->done == kRunning);
}

// E0: rows, no matrix. Unscaled y candidates, the row half of the dual objective and dual
// violation (src/pdhg/pdhg_evaluate.cpp:80-98), and |y - y_restart|^2.
__global__ void __launch_bounds__(kTileThreads) k_eval_rows0(EvalBuffers e) {
  __shared__ double scratch[kScratch];
  const Ctl* c = e.ctl;
  if (!eval_active(c)) return;
  const bool fin = c->final_mode != 0;
  const int cur = c->cur;
  const bool avg = !fin && c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const double count = static_cast<double>(c->averaged);
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // support0, viol0, support1, viol1, dy^2
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < e.m; i += gridDim.x * blockDim.x) {
    double cand[2];
    int nc = 1;
    if (fin) {
      cand[0] = e.best_y[i];
    } else {
      const double yc = e.y[cur][i];
      cand[0] = yc * e.dr[i];
      if (avg) {
        const double sum = pend ? e.y_sum[i] + yc : e.y_sum[i];
        cand[1] = (sum / count) * e.dr[i];
        nc = 2;
      }
      const double d = yc - e.y_rst[i];
      acc[4] += d * d;
    }
    const double rl = e.rl[i], ru = e.ru[i];
    for (int q = 0; q < nc; ++q) {
      const double yi = cand[q];
      e.yu[q][i] = yi;
      if (yi > 0.0) {
        if (finite_bound(ru)) acc[2 * q] += yi * ru; else acc[2 * q + 1] += yi * yi;
      } else if (yi < 0.0) {
        if (finite_bound(rl)) acc[2 * q] += yi * rl; else acc[2 * q + 1] += yi * yi;
      }
    }
  }
  double out[5];
  block_sum<5>(acc, scratch, out);
  if (threadIdx.x == 0) {
    for (int q = 0; q < 5; ++q) e.part_rows0[blockIdx.x * kEvalRowSlots + q] = out[q];
  }
}

// E1: columns over the unscaled CSC. Reduced costs d = c + A^T y of both candidates, the
// column half of the dual violation / dual objective / complementarity, the primal objective
// (src/pdhg/pdhg_evaluate.cpp:54-78,111-139) and |x - x_restart|^2.
__global__ void __launch_bounds__(kBlockThreads) k_eval_cols(EvalBuffers e) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* c = e.ctl;
  if (!eval_active(c)) return;
  const bool fin = c->final_mode != 0;
  const int cur = c->cur;
  const bool avg = !fin && c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const double count = static_cast<double>(c->averaged);
  const double* __restrict__ yu0 = e.yu[0];
  const double* __restrict__ yu1 = e.yu[1];
  // sums: viol0, bc0, pobj0, viol1, bc1, pobj1, dx^2, model objective; maxes: comp0, comp1
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double cmax[2] = {0.0, 0.0};
  auto gather = [&](int row, double v, double* a) {
    a[0] = fma(v, yu0[row], a[0]);
    if (avg) a[1] = fma(v, yu1[row], a[1]);
  };
  auto epi = [&](int j, const double* s) {
    const double cj = e.cost[j], lj = e.l[j], uj = e.u[j];
    double xc[2];
    const int nc = avg ? 2 : 1;
    if (fin) {
      xc[0] = e.best_x[j];
      acc[7] += e.col_cost[j] * xc[0];
    } else {
      const double xj = e.x[cur][j];
      xc[0] = xj * e.dc[j];
      if (avg) {
        const double sum = pend ? e.x_sum[j] + xj : e.x_sum[j];
        xc[1] = (sum / count) * e.dc[j];
      }
      const double d = xj - e.x_rst[j];
      acc[6] += d * d;
    }
    for (int q = 0; q < nc; ++q) {
      const double d = cj + s[q];
      if (q == 0) e.reduced[j] = d;
      e.xu[q][j] = xc[q];
      if (d > 0.0) {
        if (finite_bound(lj)) acc[3 * q + 1] += d * lj; else acc[3 * q] += d * d;
      } else if (d < 0.0) {
        if (finite_bound(uj)) acc[3 * q + 1] += d * uj; else acc[3 * q] += d * d;
      }
      if (lj != uj) {
        const double ls = finite_bound(lj) ? xc[q] - lj : HUGE_VAL;
        const double us = finite_bound(uj) ? uj - xc[q] : HUGE_VAL;
        cmax[q] = dmax(cmax[q], fabs(d) * dmin(ls, us));
      }
      acc[3 * q + 2] += cj * xc[q];
    }
  };
  TilePipe<double> pipe;
  pipe.setup(dsmem);
  if (!run_tiles<2, double>(pipe, e.csc, e.chunk_cols, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(c);
  }
  double out[8], mout[2];
  block_sum<8>(acc, scratch, out);
  block_max<2>(cmax, scratch, mout);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    double* p = e.part_cols + blockIdx.x * kEvalColSlots;
    for (int q = 0; q < 8; ++q) p[q] = out[q];
    p[8] = mout[0];
    p[9] = mout[1];
    __threadfence();
    s_last = atomicAdd(&c->ticket[kTicketEvalCols], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // Last block: long columns into the extra slot e.part_cols[grid_cols].
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  cmax[0] = cmax[1] = 0.0;
  run_long_rows<2>(e.csc, e.chunk_cols, epi);
  block_sum<8>(acc, scratch, out);
  block_max<2>(cmax, scratch, mout);
  if (threadIdx.x == 0) {
    double* p = e.part_cols + e.grid_cols * kEvalColSlots;
    for (int q = 0; q < 8; ++q) p[q] = out[q];
    p[8] = mout[0];
    p[9] = mout[1];
    c->ticket[kTicketEvalCols] = 0;
  }
}

__device__ Residuals assemble(double pviol, double cviol, double rviol, double bc, double support,
                              double pobj, double comp, double bound_norm, double cost_norm) {
  Residuals r;
  r.absolute_primal = sqrt(pviol);
  r.primal = r.absolute_primal / (1.0 + bound_norm);
  r.absolute_dual = sqrt(cviol + rviol);
  r.dual = r.absolute_dual / (1.0 + cost_norm);
  r.complementarity = comp;
  r.primal_objective = pobj;
  r.dual_objective = bc - support;
  const double gap = fabs(r.primal_objective - r.dual_objective);
  r.gap = gap / (1.0 + fabs(r.primal_objective) + fabs(r.dual_objective));
  r.gap_as_verified = gap / dmax(1.0, fabs(r.primal_objective));
  return r;
}

// E2: rows over the unscaled CSR. Activities of both candidates, primal violation and the
// row complementarity (src/pdhg/pdhg_evaluate.cpp:29-45,99-110). The last block assembles
// the Residuals and takes the best / stop / restart decisions (src/pdhg/pdhg.cpp:349-483).
__global__ void __launch_bounds__(kBlockThreads) k_eval_rows1(EvalBuffers e) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  __shared__ double scratch[kScratch];
  Ctl* c = e.ctl;
  if (!eval_active(c)) return;
  const bool fin = c->final_mode != 0;
  const bool avg = !fin && c->averaged > 0;
  const double* __restrict__ xu0 = e.xu[0];
  const double* __restrict__ xu1 = e.xu[1];
  double acc[2] = {0.0, 0.0};
  double cmax[2] = {0.0, 0.0};
  auto gather = [&](int col, double v, double* a) {
    a[0] = fma(v, xu0[col], a[0]);
    if (avg) a[1] = fma(v, xu1[col], a[1]);
  };
  auto epi = [&](int i, const double* s) {
    const double rl = e.rl[i], ru = e.ru[i];
    const int nc = avg ? 2 : 1;
    for (int q = 0; q < nc; ++q) {
      const double a = s[q];
      double violation = 0.0;
      if (finite_bound(rl)) violation = dmax(violation, rl - a);
      if (finite_bound(ru)) violation = dmax(violation, a - ru);
      acc[q] += violation * violation;
      if (rl != ru) {
        const double ls = finite_bound(rl) ? a - rl : HUGE_VAL;
        const double us = finite_bound(ru) ? ru - a : HUGE_VAL;
        cmax[q] = dmax(cmax[q], fabs(e.yu[q][i]) * dmin(ls, us));
      }
    }
  };
  TilePipe<double> pipe;
  pipe.setup(dsmem);
  if (!run_tiles<2, double>(pipe, e.csr, e.chunk_rows, gather, epi) &&
      threadIdx.x == 0) {
    raise_error(c);
  }
  double mout[2], sums[2];
  block_max<2>(cmax, scratch, mout);
  block_sum<2>(acc, scratch, sums);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    double* p = e.part_rows1 + blockIdx.x * kEvalRowSlots;
    p[0] = sums[0];
    p[1] = sums[1];
    p[2] = mout[0];
    p[3] = mout[1];
    __threadfence();
    s_last = atomicAdd(&c->ticket[kTicketEvalRows], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // ---- Last block: long rows, then every partial in a fixed order. ----
  acc[0] = acc[1] = 0.0;
  cmax[0] = cmax[1] = 0.0;
  run_long_rows<2>(e.csr, e.chunk_rows, epi);
  double s[15];
#pragma unroll
  for (int q = 0; q < 15; ++q) s[q] = 0.0;
  double m4[4] = {cmax[0], cmax[1], 0.0, 0.0};
  s[5] = acc[0];
  s[6] = acc[1];
  for (int b = threadIdx.x; b < e.grid_rows; b += blockDim.x) {
    for (int q = 0; q < 5; ++q) s[q] += __ldcg(e.part_rows0 + b * kEvalRowSlots + q);
    s[5] += __ldcg(e.part_rows1 + b * kEvalRowSlots + 0);
    s[6] += __ldcg(e.part_rows1 + b * kEvalRowSlots + 1);
    m4[0] = dmax(m4[0], __ldcg(e.part_rows1 + b * kEvalRowSlots + 2));
    m4[1] = dmax(m4[1], __ldcg(e.part_rows1 + b * kEvalRowSlots + 3));
  }
  for (int b = threadIdx.x; b <= e.grid_cols; b += blockDim.x) {
    for (int q = 0; q < 8; ++q) s[7 + q] += __ldcg(e.part_cols + b * kEvalColSlots + q);
    m4[2] = dmax(m4[2], __ldcg(e.part_cols + b * kEvalColSlots + 8));
    m4[3] = dmax(m4[3], __ldcg(e.part_cols + b * kEvalColSlots + 9));
  }
  double t15[15];
  block_sum<15>(s, scratch, t15);
  double t4[4];
  block_max<4>(m4, scratch, t4);
  if (threadIdx.x != 0) return;
  c->ticket[kTicketEvalRows] = 0;
  // t15: [0] support0 [1] rviol0 [2] support1 [3] rviol1 [4] dy^2 [5] pviol0 [6] pviol1
  //      [7] cviol0 [8] bc0 [9] pobj0 [10] cviol1 [11] bc1 [12] pobj1 [13] dx^2 [14] model obj
  const Residuals cur = assemble(t15[5], t15[7], t15[1], t15[8], t15[0], t15[9],
                                 dmax(t4[0], t4[2]), e.bound_norm, e.cost_norm);
  if (fin) {
    c->final_residuals = cur;
    c->model_objective = t15[14];
    return;
  }
  Residuals av;
  if (avg) {
    av = assemble(t15[6], t15[10], t15[3], t15[11], t15[2], t15[12], dmax(t4[1], t4[3]),
                  e.bound_norm, e.cost_norm);
  }
  tick_decisions(c, cur, avg ? &av : nullptr, fp64_stop_test, t15[13], t15[4], 1e-6, 1e6);
}

// E4: the vector half of the decisions: best point copy, restart anchors, zeroed sums. The
// last block to finish clears the evaluation flags, which lets the next step run.
__global__ void k_eval_apply(EvalBuffers e) {
  Ctl* c = e.ctl;
  if (c->eval_now == 0 || c->final_mode != 0) return;
  const int copy = c->copy_best;
  const bool restart = c->do_restart != 0;
  const int cur = c->cur;
  const int total = (copy == 0 && !restart) ? 0 : (e.m > e.n ? e.m : e.n);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    if (k < e.n) {
      if (copy) e.best_x[k] = e.xu[copy - 1][k];
      if (restart) {
        e.x_rst[k] = e.x[cur][k];
        e.x_sum[k] = 0.0;
      }
    }
    if (k < e.m) {
      if (copy) e.best_y[k] = e.yu[copy - 1][k];
      if (restart) {
        e.y_rst[k] = e.y[cur][k];
        e.y_sum[k] = 0.0;
      }
    }
  }
  clear_evaluation_flags(c);
}

// ---- Setup kernels (src/la/scaling.cpp) ----------------------------------------------------

// One thread per row (CSR) or column (CSC): the maximum (Ruiz) or the sum (Pock-Chambolle)
// of |a| in ascending index order -- the reference's accumulation order -- then the pass
// factor 1/sqrt(.) (1 for an empty line).
__global__ void k_line_factor(const int* ptr, const double* val, int lines, int sum_mode,
                              double* factor) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < lines; r += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      const double mag = fabs(val[k]);
      acc = sum_mode ? acc + mag : dmax(acc, mag);
    }
    factor[r] = acc > 0.0 ? 1.0 / sqrt(acc) : 1.0;
  }
}

// value <- (value * row_pass[i]) * col_pass[j], in both layouts (src/la/scaling.cpp:21-28).
__global__ void k_apply_pass(const int* ptr, const int* idx, double* val, int lines,
                             const double* line_pass, const double* other_pass, int line_is_row) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < lines; r += gridDim.x * blockDim.x) {
    const double lp = line_pass[r];
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      const double op = other_pass[idx[k]];
      val[k] = line_is_row ? (val[k] * lp) * op : (val[k] * op) * lp;
    }
  }
}

__global__ void k_mul_into(double* acc, const double* factor, int count) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < count; r += gridDim.x * blockDim.x) {
    acc[r] *= factor[r];
  }
}

// src/la/scaling.cpp:124-145.
__global__ void k_scale_vectors(int m, int n, const double* cost, const double* l,
                                const double* u, const double* rl, const double* ru,
                                const double* dr, const double* dc, double* cs, double* ls,
                                double* us, double* rls, double* rus) {
  const int total = m > n ? m : n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    // An absent bound is stored as an IEEE infinity (the reference keeps +-1e30 as is and
    // tests it with is_finite_bound each time), so the step kernels project with min/max.
    if (k < n) {
      const double d = dc[k];
      cs[k] = cost[k] * d;
      const double inv = 1.0 / d;
      ls[k] = finite_bound(l[k]) ? l[k] * inv : -HUGE_VAL;
      us[k] = finite_bound(u[k]) ? u[k] * inv : HUGE_VAL;
    }
    if (k < m) {
      const double d = dr[k];
      rls[k] = finite_bound(rl[k]) ? rl[k] * d : -HUGE_VAL;
      rus[k] = finite_bound(ru[k]) ? ru[k] * d : HUGE_VAL;
    }
  }
}

// y = A x with products summed in ascending index order per row. A block whose bounded wait
// gives up (a tile copy that never lands) sets *error and writes NaN to every row of its tile
// range and to the partials of its chunk tiles (so a long row it took part in sums to NaN):
// a product that could not be finished is never left looking like a result.
__global__ void __launch_bounds__(kBlockThreads) k_spmv(TileSet<double> a, const double* x,
                                                       double* y, double* chunk,
                                                       unsigned int* ticket,
                                                       unsigned int* error) {
  extern __shared__ __align__(16) unsigned char dsmem[];
  auto gather = [&](int col, double v, double* acc) { acc[0] = fma(v, __ldg(x + col), acc[0]); };
  auto epi = [&](int r, const double* s) { y[r] = 0.0 + s[0]; };
  TilePipe<double> pipe;
  pipe.setup(dsmem);
  if (!run_tiles<1, double>(pipe, a, chunk, gather, epi)) {
    int first, last;
    block_tile_range(a.ntiles, first, last);
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int t = first; t < last; ++t) {
      const Tile tl = a.tiles[t];
      if (tl.r1 < 0) {
        if (threadIdx.x == 0) chunk[-tl.r1 - 1] = nan;
      } else {
        for (int r = tl.r0 + static_cast<int>(threadIdx.x); r < tl.r1; r += blockDim.x) y[r] = nan;
      }
    }
    if (threadIdx.x == 0) atomicExch(error, 1u);
  }
  if (a.nlong == 0) return;
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    __threadfence();  // this block's chunk partials (written by thread 0) before the ticket
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  run_long_rows<1>(a, chunk, epi);
  if (threadIdx.x == 0) *ticket = 0;
}

__global__ void k_sumsq(const double* v, int count, double* part, double* out,
                        unsigned int* ticket) {
  __shared__ double scratch[kTileThreads / 32];
  double acc[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    acc[0] = fma(v[k], v[k], acc[0]);
  }
  double o[1];
  block_sum<1>(acc, scratch, o);
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = o[0];
    __threadfence();
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double a[1] = {0.0};
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) a[0] += __ldcg(part + b);
  block_sum<1>(a, scratch, o);
  if (threadIdx.x == 0) {
    *out = o[0];
    *ticket = 0;
  }
}

__global__ void k_div_by_sqrt(double* v, int count, const double* sq) {
  const double length = sqrt(*sq);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    v[k] /= length;
  }
}

__global__ void k_abs_minmax(const double* v, int count, double* part, double* out,
                             unsigned int* ticket) {
  __shared__ double scratch[2 * (kTileThreads / 32)];
  double mx[2] = {0.0, -HUGE_VAL};  // max |v|, max -|v| (= -min |v|)
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const double a = fabs(v[k]);
    mx[0] = dmax(mx[0], a);
    mx[1] = dmax(mx[1], -a);
  }
  double o[2];
  block_max<2>(mx, scratch, o);
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = o[0];
    part[2 * blockIdx.x + 1] = o[1];
    __threadfence();
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double a[2] = {0.0, -HUGE_VAL};
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    a[0] = dmax(a[0], __ldcg(part + 2 * b));
    a[1] = dmax(a[1], __ldcg(part + 2 * b + 1));
  }
  block_max<2>(a, scratch, o);
  if (threadIdx.x == 0) {
    out[0] = o[0];
    out[1] = count > 0 ? -o[1] : 0.0;
    *ticket = 0;
  }
}

__global__ void k_project_start(int n, const double* l, const double* u, double* x) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    x[k] = clamp_box(0.0, l[k], u[k]);
  }
}

__global__ void k_fill(double* v, int count, double value) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    v[k] = value;
  }
}

int elementwise_grid(int count) {
  int blocks = (count + 255) / 256;
  const int cap = device_sms() * 8;
  if (blocks > cap) blocks = cap;
  return blocks < 1 ? 1 : blocks;
}

constexpr int kTileSmem = TilePipe<double>::bytes();

__global__ void k_gather_values(const double* __restrict__ src, const int* __restrict__ map,
                                float* __restrict__ dst, long long count) {
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < count;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    dst[k] = static_cast<float>(src[map[k]]);
  }
}

}  // namespace

bool configure_tile_kernels() {
  const int dev = current_device();
  if (dev < 0) return false;
  std::lock_guard<std::mutex> lock(g_config_mutex);
  DeviceConfig& c = g_config[dev];
  if (c.configured) return true;
  const cudaError_t errs[] = {
      cudaFuncSetAttribute(k_primal, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           max_dynamic_smem(reinterpret_cast<const void*>(k_primal))),
      cudaFuncSetAttribute(k_dual, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           max_dynamic_smem(reinterpret_cast<const void*>(k_dual))),
      cudaFuncSetAttribute(k_eval_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem),
      cudaFuncSetAttribute(k_eval_rows1, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem),
      cudaFuncSetAttribute(k_spmv, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem)};
  for (cudaError_t e : errs) {
    if (e != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eval_rows1, kBlockThreads,
                                                    kTileSmem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  c.tile_blocks_per_sm = per_sm > 0 ? per_sm : 1;
  c.configured = true;
  return true;
}

int tile_blocks_per_sm() {
  if (!configure_tile_kernels()) return 1;
  const int dev = current_device();
  std::lock_guard<std::mutex> lock(g_config_mutex);
  return dev >= 0 ? g_config[dev].tile_blocks_per_sm : 1;
}

long long kernel_launch_count() { return g_launches; }

int fp64_window_capacity(int pass) {
  configure_tile_kernels();
  return pass == 0 ? window_capacity(reinterpret_cast<const void*>(k_primal),
                                     PrimalPipe::bytes(), sizeof(double))
                   : window_capacity(reinterpret_cast<const void*>(k_dual), DualPipe::bytes(),
                                     sizeof(double2));
}

int fp64_step_smem(int pass, int wmax) {
  return pass == 0 ? PrimalPipe::bytes() + window_bytes(wmax, sizeof(double))
                   : DualPipe::bytes() + window_bytes(wmax, sizeof(double2));
}

int fp64_step_blocks_per_sm(int pass, int smem) {
  configure_tile_kernels();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, pass == 0 ? k_primal : k_dual, kBlockThreads, static_cast<size_t>(smem)) !=
      cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return per_sm > 0 ? per_sm : 1;
}

void launch_primal_pass(const StepBuffers& b, cudaStream_t s) {
  k_primal<<<b.grid_primal, kBlockThreads, b.smem_primal, s>>>(b);
  ++g_launches;
}

void launch_dual_pass(const StepBuffers& b, cudaStream_t s) {
  k_dual<<<b.grid_dual, kBlockThreads, b.smem_dual, s>>>(b);
  ++g_launches;
}

void launch_pdhg_step(const StepBuffers& b, cudaStream_t s) {
  launch_primal_pass(b, s);
  launch_dual_pass(b, s);
}

void launch_gather_values(const double* src, const int* map, float* dst, long long count,
                          cudaStream_t s) {
  if (count <= 0) return;
  ++g_launches;
  k_gather_values<<<elementwise_grid(static_cast<int>(std::min<long long>(count, 1 << 30))),
                           256, 0, s>>>(src, map, dst, count);
}

void launch_evaluation(const EvalBuffers& e, cudaStream_t s) {
  g_launches += 4;
  k_eval_rows0<<<e.grid_rows, kTileThreads, 0, s>>>(e);
  k_eval_cols<<<e.grid_cols, kBlockThreads, kTileSmem, s>>>(e);
  k_eval_rows1<<<e.grid_rows, kBlockThreads, kTileSmem, s>>>(e);
  const int total = e.m > e.n ? e.m : e.n;
  k_eval_apply<<<elementwise_grid(total), 256, 0, s>>>(e);
}

void launch_scaling_round(int m, int n, TileSet<double> csr, TileSet<double> csc, double* csr_val,
                          double* csc_val, double* row_acc, double* col_acc, double* dr,
                          double* dc, int sum_mode, cudaStream_t s) {
  g_launches += 6;
  k_line_factor<<<elementwise_grid(m), 256, 0, s>>>(csr.ptr, csr_val, m, sum_mode, row_acc);
  k_line_factor<<<elementwise_grid(n), 256, 0, s>>>(csc.ptr, csc_val, n, sum_mode, col_acc);
  k_apply_pass<<<elementwise_grid(m), 256, 0, s>>>(csr.ptr, csr.idx, csr_val, m, row_acc, col_acc,
                                                   1);
  k_apply_pass<<<elementwise_grid(n), 256, 0, s>>>(csc.ptr, csc.idx, csc_val, n, col_acc, row_acc,
                                                   0);
  k_mul_into<<<elementwise_grid(m), 256, 0, s>>>(dr, row_acc, m);
  k_mul_into<<<elementwise_grid(n), 256, 0, s>>>(dc, col_acc, n);
}

void launch_scale_vectors(int m, int n, const double* cost, const double* l, const double* u,
                          const double* rl, const double* ru, const double* dr, const double* dc,
                          double* cs, double* ls, double* us, double* rls, double* rus,
                          cudaStream_t s) {
  ++g_launches;
  k_scale_vectors<<<elementwise_grid(m > n ? m : n), 256, 0, s>>>(m, n, cost, l, u, rl, ru, dr, dc,
                                                                  cs, ls, us, rls, rus);
}

__global__ void k_step_factors(double2* table, long long n) {
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < n;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    table[e] = step_factors(step_factor_index(e - 1));
  }
}

void launch_step_factors(double2* table, long long n, cudaStream_t s) {
  if (n <= 0) return;
  ++g_launches;
  k_step_factors<<<std::max(1, device_sms()) * 8, 256, 0, s>>>(table, n);
}

void launch_spmv(TileSet<double> a, const double* x, double* y, double* chunk,
                 unsigned int* ticket, unsigned int* error, cudaStream_t s, int grid) {
  if (a.nrows == 0) return;
  ++g_launches;
  k_spmv<<<grid, kBlockThreads, kTileSmem, s>>>(a, x, y, chunk, ticket, error);
}

namespace {

// The allocation-free product's scratch: file-scope device arrays, never cudaMalloc'd.
// g_noalloc_ticket[0] is the product's completion counter, [1] its error word.
static __device__ __align__(256) double g_noalloc_chunks[kNoAllocMaxChunks];
static __device__ __align__(256) unsigned int g_noalloc_ticket[4];

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocSlot {
  bool ready;
  double* chunks;
  unsigned int* ticket;
};
std::mutex g_noalloc_mutex;
NoAllocSlot g_noalloc_slots[kNoAllocMaxDevices];

}  // namespace

cudaError_t noalloc_scratch(int device, cudaStream_t s, double** chunks, unsigned int** ticket,
                            unsigned int** error) {
  if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocSlot& slot = g_noalloc_slots[device];
  if (!slot.ready) {
    cudaError_t err = cudaSetDevice(device);
    if (err != cudaSuccess) return err;
    void* c = nullptr;
    void* t = nullptr;
    err = cudaGetSymbolAddress(&c, g_noalloc_chunks);
    if (err != cudaSuccess) return err;
    err = cudaGetSymbolAddress(&t, g_noalloc_ticket);
    if (err != cudaSuccess) return err;
    // The completion counter must start at zero; k_spmv's last block puts it back to zero.
    // The error word starts at zero too. The chunk partials need no clearing: each is
    // written before it is read.
    err = cudaMemsetAsync(t, 0, sizeof(g_noalloc_ticket), s);
    if (err != cudaSuccess) return err;
    err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return err;
    slot.chunks = static_cast<double*>(c);
    slot.ticket = static_cast<unsigned int*>(t);
    slot.ready = true;
  }
  *chunks = slot.chunks;
  *ticket = slot.ticket;
  *error = slot.ticket + 1;
  return cudaSuccess;
}

void launch_sumsq(const double* v, int count, double* part, double* out, unsigned int* ticket,
                  cudaStream_t s, int grid) {
  ++g_launches;
  k_sumsq<<<grid, kTileThreads, 0, s>>>(v, count, part, out, ticket);
}

void launch_scale_div(double* v, int count, const double* by_sqrt_of, cudaStream_t s) {
  ++g_launches;
  k_div_by_sqrt<<<elementwise_grid(count), 256, 0, s>>>(v, count, by_sqrt_of);
}

void launch_abs_minmax(const double* v, int count, double* part, double* out,
                       unsigned int* ticket, cudaStream_t s, int grid) {
  ++g_launches;
  k_abs_minmax<<<grid, kTileThreads, 0, s>>>(v, count, part, out, ticket);
}

void launch_project_start(int n, const double* l, const double* u, double* x, cudaStream_t s) {
  ++g_launches;
  k_project_start<<<elementwise_grid(n), 256, 0, s>>>(n, l, u, x);
}

void launch_fill(double* v, int count, double value, cudaStream_t s) {
  if (count <= 0) return;
  ++g_launches;
  k_fill<<<elementwise_grid(count), 256, 0, s>>>(v, count, value);
}

}  // namespace sgb

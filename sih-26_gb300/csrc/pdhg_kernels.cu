// pdhg_kernels.cu -- the hot path of the GB300 PDHG engine.
//
// Per attempted step (src/pdhg/pdhg.cpp:220-335) there are TWO kernels:
//   k_primal  one pass over the CSC copy of Ahat: A^T y gathered per column, fused with the
//             projected primal update x' = proj(x - tau (c + A^T y)) and the primal half of
//             the movement; it also folds the previous accepted iterate into x_sum.
//   k_dual    one pass over the CSR copy: A xbar and A dx from ONE read of each row (x' and x
//             gathered, xbar = 2x' - x, dx = x' - x), fused with the Moreau dual update, the
//             dual movement and the interaction dy^T A dx; its last block sums every block's
//             partials in a fixed order and takes the step-size decision on the device.
// The evaluation tick (src/pdhg/pdhg.cpp:341-483, src/pdhg/pdhg_evaluate.cpp) is three
// fused passes over the UNSCALED values plus one vector pass; it runs only when the step
// decision asks for it and otherwise returns at once.
//
// Sparse products use row TILES: a tile is a run of consecutive rows whose nonzeros fit in
// shared memory. The block loads the tile's indices and values with coalesced accesses,
// gathers the vector entries and stages the products in shared memory; thread r then sums
// row r of the tile sequentially in ascending index order -- the order the reference's own
// SparseMatrix::multiply / transpose_multiply accumulate in (src/la/sparse.cpp:232-259), so
// the products of A x and A^T y match the reference's bits. A row with more nonzeros than a
// tile holds is summed by the whole block. Every sum of a scalar over rows or columns uses
// a fixed grid and a fixed reduction tree, so runs are bit-reproducible.
#include "common.cuh"
#include "kernels.cuh"

#include <cstdio>

namespace sgb {

namespace {

constexpr int kUnroll = kTileCap / kTileThreads;

__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }

// Visit every tile of `mat` assigned to this block. prod(k, index, value, p[NP]) fills the
// NP products of nonzero k; epi(row, s[NP]) consumes a row's sums on one thread.
template <int NP, typename Prod, typename Epi>
__device__ __forceinline__ void tile_loop(const Matrix<double>& mat, double* smem, Prod prod,
                                          Epi epi) {
  for (int t = blockIdx.x; t < mat.ntiles; t += gridDim.x) {
    const int2 tile = mat.tiles[t];
    const int k0 = mat.ptr[tile.x];
    const int k1 = mat.ptr[tile.y];
    if (k1 - k0 > kTileCap) {
      // One long row: strided over the whole block, then a block reduction.
      double acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = 0.0;
      for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        double p[NP];
        prod(k, mat.idx[k], mat.val[k], p);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] += p[q];
      }
      double out[NP];
      block_sum<NP>(acc, smem, out);
      if (threadIdx.x == 0) epi(tile.x, out);
      __syncthreads();
      continue;
    }
    int ci[kUnroll];
    double vv[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const int k = k0 + threadIdx.x + u * kTileThreads;
      if (k < k1) {
        ci[u] = __ldcs(mat.idx + k);
        vv[u] = __ldcs(mat.val + k);
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const int k = k0 + threadIdx.x + u * kTileThreads;
      if (k < k1) {
        double p[NP];
        prod(k, ci[u], vv[u], p);
#pragma unroll
        for (int q = 0; q < NP; ++q) smem[q * kTileCap + (k - k0)] = p[q];
      }
    }
    __syncthreads();
    const int r = tile.x + threadIdx.x;
    if (r < tile.y) {
      const int a = mat.ptr[r] - k0, b = mat.ptr[r + 1] - k0;
      double s[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) s[q] = 0.0;
      for (int k = a; k < b; ++k) {
#pragma unroll
        for (int q = 0; q < NP; ++q) s[q] += smem[q * kTileCap + k];
      }
      epi(r, s);
    }
    __syncthreads();
  }
}

// Block-level partial write plus "am I the last block" ticket (threadfence reduction).
template <int NV>
__device__ __forceinline__ bool publish_partials(double (&v)[NV], double* scratch, double* part,
                                                 unsigned int* ticket) {
  double out[NV];
  block_sum<NV>(v, scratch, out);
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) part[blockIdx.x * NV + q] = out[q];
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// ---- Step decision, src/pdhg/pdhg.cpp:252-335 (one thread) --------------------------------
__device__ void step_decision(Ctl* c, double movement, double interaction) {
  c->movement = movement;
  c->interaction = interaction;
  const bool no_information = interaction <= 0.0;
  const double limit = no_information ? __longlong_as_double(0x7ff0000000000000LL)
                                      : movement / interaction;
  const long long e = c->iteration + 1 > 2 ? c->iteration + 1 : 2;
  const double exponent = static_cast<double>(e);
  const double shrink = 1.0 - pow(exponent, -0.3);
  const double grow = 1.0 + pow(exponent, -0.6);
  const double proposed = dmin(shrink * limit, grow * c->eta);
  const bool accept = c->eta <= limit;
  if (accept) {
    c->cur ^= 1;
    c->iteration += 1;
    c->averaged += 1;
    c->pending_add = 1;
  } else {
    c->pending_add = 0;
  }
  if (!no_information) {
    double eta = proposed;
    eta = eta < 1e-12 ? 1e-12 : (c->eta_ceiling < eta ? c->eta_ceiling : eta);
    c->eta = eta;
  }
  c->attempts += 1;
  c->accepted = accept;
  c->no_information = no_information;
  c->eval_now = (c->iteration > 0) && ((c->iteration % 40) == 0 || no_information);
}

// ---- k_primal ----------------------------------------------------------------------------
__global__ void __launch_bounds__(kTileThreads) k_primal(StepBuffers b) {
  __shared__ double smem[kTileCap];
  Ctl* ctl = b.ctl;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // The evaluation flags of the previous step are consumed; no kernel of this step reads
    // them before the step decision sets them again.
    ctl->eval_now = 0;
    ctl->copy_best = 0;
    ctl->do_restart = 0;
  }
  if (ctl->done != kRunning) return;
  if (ctl->iteration >= ctl->iteration_limit) {  // src/pdhg/pdhg.cpp:206
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->done = kIterationLimit;
    return;
  }
  const int cur = ctl->cur;
  const double* __restrict__ x = b.x[cur];
  double* __restrict__ xn = b.x[cur ^ 1];
  const double* __restrict__ y = b.y[cur];
  const double omega = ctl->omega;
  const double tau = ctl->eta / omega;
  const bool add = ctl->pending_add != 0;
  double mv[1] = {0.0};
  tile_loop<1>(
      b.csc, smem, [&](int, int row, double v, double* p) { p[0] = v * __ldg(y + row); },
      [&](int j, const double* s) {
        const double xj = x[j];
        if (add) b.x_sum[j] += xj;
        const double gradient = b.c[j] + s[0];
        const double xnj = project(xj - tau * gradient, b.l[j], b.u[j]);
        xn[j] = xnj;
        const double d = xnj - xj;
        mv[0] += 0.5 * omega * d * d;
      });
  double out[1];
  block_sum<1>(mv, smem, out);
  if (threadIdx.x == 0) b.part_primal[blockIdx.x] = out[0];
}

// ---- k_dual ------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTileThreads) k_dual(StepBuffers b) {
  __shared__ double smem[2 * kTileCap];
  Ctl* ctl = b.ctl;
  if (ctl->done != kRunning) return;
  const int cur = ctl->cur;
  const double* __restrict__ x = b.x[cur];
  const double* __restrict__ xn = b.x[cur ^ 1];
  const double* __restrict__ y = b.y[cur];
  double* __restrict__ yn = b.y[cur ^ 1];
  const double omega = ctl->omega;
  const double sigma = ctl->eta * omega;
  const bool add = ctl->pending_add != 0;
  double acc[2] = {0.0, 0.0};  // dual movement, interaction
  tile_loop<2>(
      b.csr, smem,
      [&](int, int col, double v, double* p) {
        const double xo = __ldg(x + col), xnew = __ldg(xn + col);
        p[0] = v * (2.0 * xnew - xo);
        p[1] = v * (xnew - xo);
      },
      [&](int i, const double* s) {
        const double yi = y[i];
        if (add) b.y_sum[i] += yi;
        const double v = yi + sigma * s[0];
        const double yni = v - sigma * project(v / sigma, b.rl[i], b.ru[i]);
        yn[i] = yni;
        const double d = yni - yi;
        acc[0] += 0.5 * d * d / omega;
        acc[1] += d * s[1];
      });
  if (!publish_partials<2>(acc, smem, b.part_dual, &ctl->ticket[0])) return;
  // Last block: fixed-order sums of every block's partials, then the step decision.
  double a[3] = {0.0, 0.0, 0.0};
  for (int q = threadIdx.x; q < b.grid_primal; q += blockDim.x) a[0] += ldcg(b.part_primal + q);
  for (int q = threadIdx.x; q < b.grid_dual; q += blockDim.x) {
    a[1] += ldcg(b.part_dual + 2 * q);
    a[2] += ldcg(b.part_dual + 2 * q + 1);
  }
  double out[3];
  block_sum<3>(a, smem, out);
  if (threadIdx.x == 0) {
    ctl->ticket[0] = 0;
    step_decision(ctl, out[0] + out[1], fabs(out[2]));
  }
}

// ---- Evaluation ----------------------------------------------------------------------------
__device__ __forceinline__ bool eval_active(const Ctl* c) {
  return c->final_mode != 0 || (c->eval_now != 0 && c->done == kRunning);
}

// E0: rows, no matrix. Unscaled y candidates, the row half of the dual objective and dual
// violation (src/pdhg/pdhg_evaluate.cpp:80-98), and |y - y_restart|^2.
__global__ void __launch_bounds__(kTileThreads) k_eval_rows0(EvalBuffers e) {
  __shared__ double scratch[8 * (kTileThreads / 32)];
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
    for (int q = 0; q < 5; ++q) e.part_rows0[blockIdx.x * 8 + q] = out[q];
  }
}

// E1: columns over the unscaled CSC. Reduced costs d = c + A^T y of both candidates, the
// column half of the dual violation / dual objective / complementarity, the primal objective
// (src/pdhg/pdhg_evaluate.cpp:54-78,111-139) and |x - x_restart|^2.
__global__ void __launch_bounds__(kTileThreads) k_eval_cols(EvalBuffers e) {
  __shared__ double smem[2 * kTileCap];
  const Ctl* c = e.ctl;
  if (!eval_active(c)) return;
  const bool fin = c->final_mode != 0;
  const int cur = c->cur;
  const bool avg = !fin && c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const double count = static_cast<double>(c->averaged);
  const double* yu0 = e.yu[0];
  const double* yu1 = e.yu[1];
  // sums: viol0, bc0, pobj0, viol1, bc1, pobj1, dx^2, model objective; maxes: comp0, comp1
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double cmax[2] = {0.0, 0.0};
  tile_loop<2>(
      e.csc, smem,
      [&](int, int row, double v, double* p) {
        p[0] = v * yu0[row];
        p[1] = avg ? v * yu1[row] : 0.0;
      },
      [&](int j, const double* s) {
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
      });
  double out[8];
  block_sum<8>(acc, smem, out);
  double mout[2];
  block_max<2>(cmax, smem, mout);
  if (threadIdx.x == 0) {
    for (int q = 0; q < 8; ++q) e.part_cols[blockIdx.x * 16 + q] = out[q];
    e.part_cols[blockIdx.x * 16 + 8] = mout[0];
    e.part_cols[blockIdx.x * 16 + 9] = mout[1];
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
__global__ void __launch_bounds__(kTileThreads) k_eval_rows1(EvalBuffers e) {
  __shared__ double smem[2 * kTileCap];
  Ctl* c = e.ctl;
  if (!eval_active(c)) return;
  const bool fin = c->final_mode != 0;
  const bool avg = !fin && c->averaged > 0;
  const double* xu0 = e.xu[0];
  const double* xu1 = e.xu[1];
  double acc[2] = {0.0, 0.0};
  double cmax[2] = {0.0, 0.0};
  tile_loop<2>(
      e.csr, smem,
      [&](int, int col, double v, double* p) {
        p[0] = v * xu0[col];
        p[1] = avg ? v * xu1[col] : 0.0;
      },
      [&](int i, const double* s) {
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
      });
  double mout[2];
  block_max<2>(cmax, smem, mout);
  double packed[4] = {acc[0], acc[1], 0.0, 0.0};
  __shared__ double mx[2];
  if (threadIdx.x == 0) {
    mx[0] = mout[0];
    mx[1] = mout[1];
  }
  __syncthreads();
  // part_rows1 holds [pviol0, pviol1, comp0, comp1] per block; maxima are written directly.
  if (threadIdx.x == 0) {
    e.part_rows1[blockIdx.x * 8 + 2] = mx[0];
    e.part_rows1[blockIdx.x * 8 + 3] = mx[1];
  }
  double two[2] = {packed[0], packed[1]};
  double sums[2];
  block_sum<2>(two, smem, sums);
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    e.part_rows1[blockIdx.x * 8 + 0] = sums[0];
    e.part_rows1[blockIdx.x * 8 + 1] = sums[1];
    __threadfence();
    const unsigned int t = atomicAdd(&c->ticket[1], 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();

  // ---- Last block: combine the three passes in a fixed order. ----
  double s[15];
#pragma unroll
  for (int q = 0; q < 15; ++q) s[q] = 0.0;
  double m4[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < e.grid_rows; b += blockDim.x) {
    for (int q = 0; q < 5; ++q) s[q] += ldcg(e.part_rows0 + b * 8 + q);
    s[5] += ldcg(e.part_rows1 + b * 8 + 0);
    s[6] += ldcg(e.part_rows1 + b * 8 + 1);
    m4[0] = dmax(m4[0], ldcg(e.part_rows1 + b * 8 + 2));
    m4[1] = dmax(m4[1], ldcg(e.part_rows1 + b * 8 + 3));
  }
  for (int b = threadIdx.x; b < e.grid_cols; b += blockDim.x) {
    for (int q = 0; q < 8; ++q) s[7 + q] += ldcg(e.part_cols + b * 16 + q);
    m4[2] = dmax(m4[2], ldcg(e.part_cols + b * 16 + 8));
    m4[3] = dmax(m4[3], ldcg(e.part_cols + b * 16 + 9));
  }
  double t15[15];
  block_sum<15>(s, smem, t15);
  double t4[4];
  block_max<4>(m4, smem, t4);
  if (threadIdx.x != 0) return;
  c->ticket[1] = 0;
  // t15: [0] support0 [1] rviol0 [2] support1 [3] rviol1 [4] dy^2 [5] pviol0 [6] pviol1
  //      [7] cviol0 [8] bc0 [9] pobj0 [10] cviol1 [11] bc1 [12] pobj1 [13] dx^2 [14] model obj
  const Residuals cur = assemble(t15[5], t15[7], t15[1], t15[8], t15[0], t15[9],
                                 dmax(t4[0], t4[2]), e.bound_norm, e.cost_norm);
  if (fin) {
    c->final_residuals = cur;
    c->model_objective = t15[14];
    return;
  }
  c->evaluations += 1;
  Residuals chosen = cur;
  int which = 1;
  if (avg) {
    const Residuals av = assemble(t15[6], t15[10], t15[3], t15[11], t15[2], t15[12],
                                  dmax(t4[1], t4[3]), e.bound_norm, e.cost_norm);
    if (worst(av) < worst(cur)) {
      chosen = av;
      which = 2;
    }
  }
  int copy = 0;
  if (worst(chosen) < worst(c->best)) {
    c->best = chosen;
    copy = which;
  }
  {
    const long long slot = c->log_count % kLogRing;
    c->log[slot].iteration = c->iteration;
    c->log[slot].primal_objective = chosen.primal_objective;
    c->log[slot].primal = chosen.primal;
    c->log[slot].dual = chosen.dual;
    c->log[slot].gap = chosen.gap;
    c->log_count += 1;
  }
  if (meets_request(chosen, c->tolerance) &&
      (c->stop_at_request || meets_project_standard(chosen))) {
    c->best = chosen;
    c->copy_best = which;
    c->done = kConverged;
    return;
  }
  c->copy_best = copy;
  if (c->use_restarts) {
    const double kkt = worst(chosen);
    const long long since = c->iteration - c->last_restart;
    const bool sufficient = kkt <= 0.2 * c->restart_kkt;
    const long long f36 = static_cast<long long>(0.36 * static_cast<double>(c->iteration));
    const bool artificial = since >= (f36 > 40 ? f36 : 40);
    if (sufficient || artificial) {
      const double dx_norm = sqrt(t15[13]);
      const double dy_norm = sqrt(t15[4]);
      if (dx_norm > 1e-12 && dy_norm > 1e-12) {
        const double theta = 0.5;
        double omega = exp(theta * log(dy_norm / dx_norm) + (1.0 - theta) * log(c->omega));
        omega = omega < 1e-6 ? 1e-6 : (1e6 < omega ? 1e6 : omega);
        c->omega = omega;
      }
      c->do_restart = 1;
      c->averaged = 0;
      c->pending_add = 0;
      c->restart_kkt = kkt;
      c->last_restart = c->iteration;
      c->restarts += 1;
    }
  }
}

// E4: the vector half of the decisions: best point copy, restart anchors, zeroed sums.
__global__ void k_eval_apply(EvalBuffers e) {
  const Ctl* c = e.ctl;
  if (c->eval_now == 0 || c->final_mode != 0) return;
  const int copy = c->copy_best;
  const bool restart = c->do_restart != 0;
  if (copy == 0 && !restart) return;
  const int cur = c->cur;
  const int total = e.m > e.n ? e.m : e.n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    if (k < e.n) {
      if (copy) e.best_x[k] = e.xu[copy - 1][k];
      if (restart) {
        const_cast<double*>(e.x_rst)[k] = e.x[cur][k];
        const_cast<double*>(e.x_sum)[k] = 0.0;
      }
    }
    if (k < e.m) {
      if (copy) e.best_y[k] = e.yu[copy - 1][k];
      if (restart) {
        const_cast<double*>(e.y_rst)[k] = e.y[cur][k];
        const_cast<double*>(e.y_sum)[k] = 0.0;
      }
    }
  }
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
    if (k < n) {
      const double d = dc[k];
      cs[k] = cost[k] * d;
      const double inv = 1.0 / d;
      ls[k] = finite_bound(l[k]) ? l[k] * inv : l[k];
      us[k] = finite_bound(u[k]) ? u[k] * inv : u[k];
    }
    if (k < m) {
      const double d = dr[k];
      rls[k] = finite_bound(rl[k]) ? rl[k] * d : rl[k];
      rus[k] = finite_bound(ru[k]) ? ru[k] * d : ru[k];
    }
  }
}

__global__ void __launch_bounds__(kTileThreads) k_spmv(Matrix<double> a, const double* x,
                                                       double* y) {
  __shared__ double smem[kTileCap];
  tile_loop<1>(
      a, smem, [&](int, int col, double v, double* p) { p[0] = v * __ldg(x + col); },
      [&](int r, const double* s) { y[r] = 0.0 + s[0]; });
}

__global__ void k_sumsq(const double* v, int count, double* part, double* out,
                        unsigned int* ticket) {
  __shared__ double scratch[kTileThreads / 32];
  double acc[1] = {0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    acc[0] += v[k] * v[k];
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
    x[k] = project(0.0, l[k], u[k]);
  }
}

__global__ void k_fill(double* v, int count, double value) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    v[k] = value;
  }
}

int g_tile_blocks_per_sm = 0;
int g_num_sms = 0;

int elementwise_grid(int count) {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int blocks = (count + 255) / 256;
  const int cap = g_num_sms * 8;
  if (blocks > cap) blocks = cap;
  return blocks < 1 ? 1 : blocks;
}

unsigned int* g_scratch_ticket = nullptr;

unsigned int* scratch_ticket() {
  if (g_scratch_ticket == nullptr) {
    cudaMalloc(&g_scratch_ticket, sizeof(unsigned int));
    cudaMemset(g_scratch_ticket, 0, sizeof(unsigned int));
  }
  return g_scratch_ticket;
}

}  // namespace

int tile_blocks_per_sm() {
  if (g_tile_blocks_per_sm == 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dual, kTileThreads, 0);
    g_tile_blocks_per_sm = per_sm > 0 ? per_sm : 1;
  }
  return g_tile_blocks_per_sm;
}

void launch_pdhg_step(const StepBuffers& b, cudaStream_t s) {
  k_primal<<<b.grid_primal, kTileThreads, 0, s>>>(b);
  k_dual<<<b.grid_dual, kTileThreads, 0, s>>>(b);
}

void launch_evaluation(const EvalBuffers& e, const StepBuffers& b, cudaStream_t s) {
  (void)b;
  k_eval_rows0<<<e.grid_rows, kTileThreads, 0, s>>>(e);
  k_eval_cols<<<e.grid_cols, kTileThreads, 0, s>>>(e);
  k_eval_rows1<<<e.grid_rows, kTileThreads, 0, s>>>(e);
  const int total = e.m > e.n ? e.m : e.n;
  k_eval_apply<<<elementwise_grid(total), 256, 0, s>>>(e);
}

void launch_scaling_round(int m, int n, Matrix<double> csr, Matrix<double> csc, double* csr_val,
                          double* csc_val, double* row_acc, double* col_acc, double* dr,
                          double* dc, int sum_mode, cudaStream_t s) {
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
  k_scale_vectors<<<elementwise_grid(m > n ? m : n), 256, 0, s>>>(m, n, cost, l, u, rl, ru, dr, dc,
                                                                  cs, ls, us, rls, rus);
}

void launch_spmv(Matrix<double> a, const double* x, double* y, cudaStream_t s, int grid) {
  if (a.nrows == 0) return;
  k_spmv<<<grid, kTileThreads, 0, s>>>(a, x, y);
}

void launch_sumsq(const double* v, int count, double* part, double* out, cudaStream_t s,
                  int grid) {
  k_sumsq<<<grid, kTileThreads, 0, s>>>(v, count, part, out, scratch_ticket());
}

void launch_scale_div(double* v, int count, const double* by_sqrt_of, cudaStream_t s) {
  k_div_by_sqrt<<<elementwise_grid(count), 256, 0, s>>>(v, count, by_sqrt_of);
}

void launch_abs_minmax(const double* v, int count, double* part, double* out, cudaStream_t s,
                       int grid) {
  k_abs_minmax<<<grid, kTileThreads, 0, s>>>(v, count, part, out, scratch_ticket());
}

void launch_project_start(int n, const double* l, const double* u, double* x, cudaStream_t s) {
  k_project_start<<<elementwise_grid(n), 256, 0, s>>>(n, l, u, x);
}

void launch_fill(double* v, int count, double value, cudaStream_t s) {
  if (count <= 0) return;
  k_fill<<<elementwise_grid(count), 256, 0, s>>>(v, count, value);
}

}  // namespace sgb

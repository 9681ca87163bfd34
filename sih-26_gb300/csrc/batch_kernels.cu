// batch_kernels.cu -- the persistent batched PDHG (see batch.cuh).
//
// Both launches are persistent: every block draws work items (a matrix, then an LP) from an
// atomic counter until none are left. Inside a block the arithmetic is the single-LP
// engine's, item for item: the scaling passes of src/la/scaling.cpp:14-159, the power
// iteration of :161-194, the primal and dual steps of src/pdhg/pdhg.cpp:226-247 (unfused
// where the reference rounds twice), the step-size rule, the evaluation of
// src/pdhg/pdhg_evaluate.cpp:19-139 for the current and the average candidate, the best
// point, the restart and primal-weight update and the stopping test (decisions.cuh), and
// the report of src/pdhg/pdhg.cpp:487-567. Sums are per-thread FMA chains in index order,
// combined by block_sum: deterministic, like the single-LP engine's, but in a different
// order, so the two agree to rounding, not bit for bit.
#include <cuda_runtime.h>

#include <algorithm>

#include "batch.cuh"
#include "common.cuh"
#include "decisions.cuh"
#include "kernels.cuh"
#include "sankhya_gb300.h"

namespace sgb {
namespace {

constexpr int kBScratch = 16 * (kBatchMaxThreads / 32);
// A dual change d is accepted as a Farkas certificate when its value (see batch_farkas) is
// above this share of the magnitude of the terms that make it up, at two evaluations in a
// row. For a feasible LP the value is <= 0 in exact arithmetic.
constexpr double kFarkasShare = 1e-6;

// Next work item of a persistent launch (-1: none left). Every thread of the block calls it.
__device__ int next_item(unsigned int* counter, int count, int* s_item) {
  __syncthreads();  // every thread has read the previous item
  if (threadIdx.x == 0) *s_item = static_cast<int>(atomicAdd(counter, 1u));
  __syncthreads();
  const int item = *s_item;
  return item < count ? item : -1;
}

// ---- Scaling and norm estimate, one block per distinct matrix ------------------------------
__global__ void __launch_bounds__(kBatchThreads) k_batch_scale(BatchBuffers b) {
  __shared__ double scratch[kBScratch];
  __shared__ int s_item;
  __shared__ int s_zero;
  const int T = blockDim.x, t = threadIdx.x;
  for (int mi = next_item(&b.queue[0], b.nmatrices, &s_item); mi >= 0;
       mi = next_item(&b.queue[0], b.nmatrices, &s_item)) {
    const BatchMatrix M = b.matrices[mi];
    const int m = M.m, n = M.n;
    const long long nnz = M.nnz;
    const int* cp = b.csc_ptr + M.cptr;
    const int* ci = b.csc_idx + M.nz;
    const int* rp = b.csr_ptr + M.rptr;
    const int* ri = b.csr_idx + M.nz;
    double* cv = b.csc_s + M.nz;
    double* rv = b.csr_s + M.nz;
    double* dr = b.dr + M.row;
    double* dc = b.dc + M.col;
    double* racc = b.row_acc + M.row;
    double* cacc = b.col_acc + M.col;
    for (long long k = t; k < nnz; k += T) {
      cv[k] = b.csc_raw[M.nz + k];
      rv[k] = b.csr_raw[M.nz + k];
    }
    for (int i = t; i < m; i += T) dr[i] = 1.0;
    for (int j = t; j < n; j += T) dc[j] = 1.0;
    __syncthreads();
    // 10 Ruiz rounds (infinity norm), then one Pock-Chambolle round (1-norm).
    for (int pass = 0; pass < 11; ++pass) {
      const bool sum_mode = pass == 10;
      for (int r = t; r < m; r += T) {
        double acc = 0.0;
        for (int k = rp[r]; k < rp[r + 1]; ++k) {
          const double mag = fabs(rv[k]);
          acc = sum_mode ? acc + mag : dmax(acc, mag);
        }
        racc[r] = acc > 0.0 ? 1.0 / sqrt(acc) : 1.0;
      }
      for (int c = t; c < n; c += T) {
        double acc = 0.0;
        for (int k = cp[c]; k < cp[c + 1]; ++k) {
          const double mag = fabs(cv[k]);
          acc = sum_mode ? acc + mag : dmax(acc, mag);
        }
        cacc[c] = acc > 0.0 ? 1.0 / sqrt(acc) : 1.0;
      }
      __syncthreads();
      for (int r = t; r < m; r += T) {
        const double lp = racc[r];
        for (int k = rp[r]; k < rp[r + 1]; ++k) rv[k] = (rv[k] * lp) * cacc[ri[k]];
        dr[r] *= lp;
      }
      for (int c = t; c < n; c += T) {
        const double lp = cacc[c];
        for (int k = cp[c]; k < cp[c + 1]; ++k) cv[k] = (cv[k] * racc[ci[k]]) * lp;
        dc[c] *= lp;
      }
      __syncthreads();
    }
    // The power iteration on A'A from the host-drawn start vector (mt19937(seed + 1)).
    double* v = b.power_v + M.col;
    double* av = b.power_av + M.row;
    double norm = 0.0;
    if (t == 0) s_zero = (m == 0 || n == 0 || nnz == 0) ? 1 : 0;
    __syncthreads();
    for (int step = 0; step < 30 && !s_zero; ++step) {
      double a[1] = {0.0}, o[1];
      for (int j = t; j < n; j += T) a[0] = fma(v[j], v[j], a[0]);
      block_sum<1>(a, scratch, o);
      __shared__ double s_len;
      if (t == 0) {
        s_len = sqrt(o[0]);
        if (s_len == 0.0) s_zero = 1;
      }
      __syncthreads();
      if (s_zero) break;
      const double len = s_len;
      for (int j = t; j < n; j += T) v[j] /= len;
      __syncthreads();
      for (int r = t; r < m; r += T) {
        double acc = 0.0;
        for (int k = rp[r]; k < rp[r + 1]; ++k) acc = fma(rv[k], v[ri[k]], acc);
        av[r] = 0.0 + acc;
      }
      __syncthreads();
      for (int c = t; c < n; c += T) {
        double acc = 0.0;
        for (int k = cp[c]; k < cp[c + 1]; ++k) acc = fma(cv[k], av[ci[k]], acc);
        v[c] = 0.0 + acc;
      }
      __syncthreads();
      a[0] = 0.0;
      for (int j = t; j < n; j += T) a[0] = fma(v[j], v[j], a[0]);
      block_sum<1>(a, scratch, o);
      if (t == 0) norm = sqrt(sqrt(o[0]));
    }
    double mx[2] = {0.0, -HUGE_VAL};
    for (long long k = t; k < nnz; k += T) {
      const double a = fabs(cv[k]);
      mx[0] = dmax(mx[0], a);
      mx[1] = dmax(mx[1], -a);
      if (b.csc_f != nullptr) {  // the mixed method's FP32 copies
        b.csc_f[M.nz + k] = static_cast<float>(cv[k]);
        b.csr_f[M.nz + k] = static_cast<float>(rv[k]);
      }
    }
    double mo[2];
    block_max<2>(mx, scratch, mo);
    if (t == 0) {
      BatchMatrix& out = b.matrices_out[mi];
      out.spectral_norm = (s_zero || !(norm > 0.0)) ? 1.0 : norm * 1.01;
      out.scaled_max_abs = mo[0];
      out.scaled_min_abs = nnz > 0 ? -mo[1] : 0.0;
    }
  }
}

// ---- One LP, one block ---------------------------------------------------------------------
struct LpView {
  int m, n;
  const int *cp, *ci, *rp, *ri;
  const double *csv, *rsv;     // scaled values
  const double *craw, *rraw;   // unscaled values
  const double *dr, *dc;
  const double *cost, *col_cost, *l, *u, *rl, *ru;
  double *cs, *ls, *us, *rls, *rus;
  double *x[2], *x_sum, *x_rst, *xu[2], *best_x, *reduced;
  double2* xd;
  double *y[2], *y_sum, *y_rst, *yu[2], *best_y;
  double* ray;
  double bound_norm, cost_norm;
  int lanes;  // threads that share a row or column in the matrix passes (a power of two)
};

// The lanes of a line group (`lanes` consecutive threads, aligned inside a warp) add their
// partial sums in a fixed xor tree; every lane receives the total. Every thread of the warp
// calls it (the line loops below run the same number of iterations in every thread).
template <typename V>
__device__ __forceinline__ V lanes_sum(V s, int lanes) {
  for (int o = lanes >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

__device__ LpView make_view(const BatchBuffers& b, const BatchInstance& I, const BatchMatrix& M) {
  LpView v;
  v.m = I.m;
  v.n = I.n;
  v.cp = b.csc_ptr + M.cptr;
  v.ci = b.csc_idx + M.nz;
  v.rp = b.csr_ptr + M.rptr;
  v.ri = b.csr_idx + M.nz;
  v.csv = b.csc_s + M.nz;
  v.rsv = b.csr_s + M.nz;
  v.craw = b.csc_raw + M.nz;
  v.rraw = b.csr_raw + M.nz;
  v.dr = b.dr + M.row;
  v.dc = b.dc + M.col;
  const long long c = I.col, r = I.row;
  v.cost = b.cost + c;
  v.col_cost = b.col_cost + c;
  v.l = b.l + c;
  v.u = b.u + c;
  v.rl = b.rl + r;
  v.ru = b.ru + r;
  v.cs = b.cs + c;
  v.ls = b.ls + c;
  v.us = b.us + c;
  v.rls = b.rls + r;
  v.rus = b.rus + r;
  v.x[0] = b.x0 + c;
  v.x[1] = b.x1 + c;
  v.x_sum = b.x_sum + c;
  v.x_rst = b.x_rst + c;
  v.xu[0] = b.xu0 + c;
  v.xu[1] = b.xu1 + c;
  v.best_x = b.best_x + c;
  v.reduced = b.reduced + c;
  v.xd = b.xd + c;
  v.y[0] = b.y0 + r;
  v.y[1] = b.y1 + r;
  v.y_sum = b.y_sum + r;
  v.y_rst = b.y_rst + r;
  v.yu[0] = b.yu0 + r;
  v.yu[1] = b.yu1 + r;
  v.best_y = b.best_y + r;
  v.ray = b.ray + r;
  v.bound_norm = I.bound_norm;
  v.cost_norm = I.cost_norm;
  v.lanes = b.lanes > 0 ? b.lanes : 1;
  return v;
}

// src/pdhg/pdhg.cpp:424-425, or relative KKT alone (stop_rule 1).
__device__ bool batch_stop_test(const Ctl* c, const Residuals& r) {
  return c->stop_rule == 1 ? worst(r) <= c->tolerance
                           : meets_request(r, c->tolerance) &&
                                 (c->stop_at_request || meets_project_standard(r));
}

// The primal step over the LP's columns (k_primal's arithmetic).
__device__ void b_primal(const LpView& v, Ctl* c, double* scratch) {
  const int T = blockDim.x;
  const int cur = c->cur;
  const double* x = v.x[cur];
  double* xn = v.x[cur ^ 1];
  const double* y = v.y[cur];
  const double omega = c->omega;
  const double tau = c->eta / omega;
  const bool add = c->pending_add != 0;
  double mv[1] = {0.0};
  // `lanes` threads per column: lane s sums entries s, s + lanes, ... in order.
  const int L = v.lanes, G = T / L, sub = threadIdx.x & (L - 1);
  for (int base = 0; base < v.n; base += G) {
    const int j = base + static_cast<int>(threadIdx.x) / L;
    double acc = 0.0;
    if (j < v.n) {
      for (int k = v.cp[j] + sub; k < v.cp[j + 1]; k += L) acc = fma(v.csv[k], y[v.ci[k]], acc);
    }
    acc = lanes_sum(acc, L);
    if (j >= v.n || sub != 0) continue;
    const double xj = x[j];
    if (add) v.x_sum[j] += xj;
    const double gradient = v.cs[j] + acc;
    const double xnj = clamp_box(__dsub_rn(xj, __dmul_rn(tau, gradient)), v.ls[j], v.us[j]);
    xn[j] = xnj;
    const double d = xnj - xj;
    v.xd[j] = make_double2(fma(2.0, xnj, -xj), d);
    mv[0] = fma(d, d, mv[0]);
  }
  double out[1];
  block_sum<1>(mv, scratch, out);
  if (threadIdx.x == 0) c->mv_primal = 0.5 * omega * out[0];
  __syncthreads();
}

// The dual step over the LP's rows (k_dual's arithmetic) and the step decision.
__device__ void b_dual(const LpView& v, Ctl* c, double* scratch) {
  const int T = blockDim.x;
  const int cur = c->cur;
  const double* y = v.y[cur];
  double* yn = v.y[cur ^ 1];
  const double omega = c->omega;
  const double sigma = c->eta * omega;
  const bool add = c->pending_add != 0;
  double acc2[2] = {0.0, 0.0};
  const int L = v.lanes, G = T / L, sub = threadIdx.x & (L - 1);
  for (int base = 0; base < v.m; base += G) {
    const int i = base + static_cast<int>(threadIdx.x) / L;
    double s0 = 0.0, s1 = 0.0;
    if (i < v.m) {
      for (int k = v.rp[i] + sub; k < v.rp[i + 1]; k += L) {
        const double2 p = v.xd[v.ri[k]];
        s0 = fma(v.rsv[k], p.x, s0);
        s1 = fma(v.rsv[k], p.y, s1);
      }
    }
    s0 = lanes_sum(s0, L);
    s1 = lanes_sum(s1, L);
    if (i >= v.m || sub != 0) continue;
    const double yi = y[i];
    if (add) v.y_sum[i] += yi;
    const double rl = v.rls[i], ru = v.rus[i];
    const double vv = __dadd_rn(yi, __dmul_rn(sigma, s0));
    const double p = rl == ru ? rl : clamp_box(vv / sigma, rl, ru);
    const double yni = __dsub_rn(vv, __dmul_rn(sigma, p));
    yn[i] = yni;
    const double d = yni - yi;
    acc2[0] = fma(d, d, acc2[0]);
    acc2[1] = fma(d, s1, acc2[1]);
  }
  double tot[2];
  block_sum<2>(acc2, scratch, tot);
  if (threadIdx.x == 0 && c->done == kRunning) {
    const double movement = c->mv_primal + (0.5 * tot[0]) / omega;
    step_decision(c, movement, fabs(tot[1]));
  }
  __syncthreads();
}

__device__ Residuals b_assemble(double pviol, double cviol, double rviol, double bc,
                                double support, double pobj, double comp, double bound_norm,
                                double cost_norm) {
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

// The evaluation of the current and average candidates (or, fin, of the best point), with
// the tick decisions; the k_eval_rows0 / k_eval_cols / k_eval_rows1 passes of the single-LP
// engine in one block. Thread 0 ends with the decisions taken (or the final residuals).
__device__ void b_evaluate(const LpView& v, Ctl* c, double* scratch, bool fin) {
  const int T = blockDim.x, t = threadIdx.x;
  const int cur = c->cur;
  const bool avg = !fin && c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const double count = static_cast<double>(c->averaged);
  const int nc = avg ? 2 : 1;
  // s: [0] support0 [1] rviol0 [2] support1 [3] rviol1 [4] dy^2 [5] pviol0 [6] pviol1
  //    [7] cviol0 [8] bc0 [9] pobj0 [10] cviol1 [11] bc1 [12] pobj1 [13] dx^2 [14] model obj
  double s[15];
#pragma unroll
  for (int q = 0; q < 15; ++q) s[q] = 0.0;
  double mx[4] = {0.0, 0.0, 0.0, 0.0};  // row comp 0/1, column comp 0/1
  for (int i = t; i < v.m; i += T) {
    double cand[2];
    if (fin) {
      cand[0] = v.best_y[i];
    } else {
      const double yc = v.y[cur][i];
      cand[0] = yc * v.dr[i];
      if (avg) {
        const double sum = pend ? v.y_sum[i] + yc : v.y_sum[i];
        cand[1] = (sum / count) * v.dr[i];
      }
      const double d = yc - v.y_rst[i];
      s[4] += d * d;
    }
    const double rl = v.rl[i], ru = v.ru[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      const double yi = cand[q];
      v.yu[q][i] = yi;
      if (yi > 0.0) {
        if (finite_bound(ru)) s[2 * q] += yi * ru; else s[2 * q + 1] += yi * yi;
      } else if (yi < 0.0) {
        if (finite_bound(rl)) s[2 * q] += yi * rl; else s[2 * q + 1] += yi * yi;
      }
    }
  }
  __syncthreads();
  const int L = v.lanes, G = T / L, sub = t & (L - 1);
  for (int base = 0; base < v.n; base += G) {
    const int j = base + t / L;
    double sq[2] = {0.0, 0.0};
    if (j < v.n) {
      for (int k = v.cp[j] + sub; k < v.cp[j + 1]; k += L) {
        const int row = v.ci[k];
        sq[0] = fma(v.craw[k], v.yu[0][row], sq[0]);
        if (avg) sq[1] = fma(v.craw[k], v.yu[1][row], sq[1]);
      }
    }
    sq[0] = lanes_sum(sq[0], L);
    sq[1] = lanes_sum(sq[1], L);
    if (j >= v.n || sub != 0) continue;
    const double cj = v.cost[j], lj = v.l[j], uj = v.u[j];
    double xc[2];
    if (fin) {
      xc[0] = v.best_x[j];
      s[14] += v.col_cost[j] * xc[0];
    } else {
      const double xj = v.x[cur][j];
      xc[0] = xj * v.dc[j];
      if (avg) {
        const double sum = pend ? v.x_sum[j] + xj : v.x_sum[j];
        xc[1] = (sum / count) * v.dc[j];
      }
      const double d = xj - v.x_rst[j];
      s[13] += d * d;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      const double d = cj + sq[q];
      if (q == 0) v.reduced[j] = d;
      v.xu[q][j] = xc[q];
      double* cs3 = s + 7 + 3 * q;  // cviol, bc, pobj of candidate q
      if (d > 0.0) {
        if (finite_bound(lj)) cs3[1] += d * lj; else cs3[0] += d * d;
      } else if (d < 0.0) {
        if (finite_bound(uj)) cs3[1] += d * uj; else cs3[0] += d * d;
      }
      if (lj != uj) {
        const double ls = finite_bound(lj) ? xc[q] - lj : HUGE_VAL;
        const double us = finite_bound(uj) ? uj - xc[q] : HUGE_VAL;
        mx[2 + q] = dmax(mx[2 + q], fabs(d) * dmin(ls, us));
      }
      cs3[2] += cj * xc[q];
    }
  }
  __syncthreads();
  for (int base = 0; base < v.m; base += G) {
    const int i = base + t / L;
    double a[2] = {0.0, 0.0};
    if (i < v.m) {
      for (int k = v.rp[i] + sub; k < v.rp[i + 1]; k += L) {
        const int col = v.ri[k];
        a[0] = fma(v.rraw[k], v.xu[0][col], a[0]);
        if (avg) a[1] = fma(v.rraw[k], v.xu[1][col], a[1]);
      }
    }
    a[0] = lanes_sum(a[0], L);
    a[1] = lanes_sum(a[1], L);
    if (i >= v.m || sub != 0) continue;
    const double rl = v.rl[i], ru = v.ru[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      double violation = 0.0;
      if (finite_bound(rl)) violation = dmax(violation, rl - a[q]);
      if (finite_bound(ru)) violation = dmax(violation, a[q] - ru);
      s[5 + q] += violation * violation;
      if (rl != ru) {
        const double ls = finite_bound(rl) ? a[q] - rl : HUGE_VAL;
        const double us = finite_bound(ru) ? ru - a[q] : HUGE_VAL;
        mx[q] = dmax(mx[q], fabs(v.yu[q][i]) * dmin(ls, us));
      }
    }
  }
  double t15[15], t4[4];
  block_sum<15>(s, scratch, t15);
  block_max<4>(mx, scratch, t4);
  if (t == 0) {
    const Residuals rc = b_assemble(t15[5], t15[7], t15[1], t15[8], t15[0], t15[9],
                                    dmax(t4[0], t4[2]), v.bound_norm, v.cost_norm);
    if (fin) {
      c->final_residuals = rc;
      c->model_objective = t15[14];
    } else {
      Residuals ra;
      if (avg) {
        ra = b_assemble(t15[6], t15[10], t15[3], t15[11], t15[2], t15[12], dmax(t4[1], t4[3]),
                        v.bound_norm, v.cost_norm);
      }
      tick_decisions(c, rc, avg ? &ra : nullptr, batch_stop_test, t15[13], t15[4], 1e-6, 1e6);
    }
  }
  __syncthreads();
}

// Farkas test of the dual change d = Dr (y - y_restart): with r = A' d (unscaled),
//   value = sum_j min over [l_j, u_j] of r_j x_j  -  sum_i max over [rl_i, ru_i] of d_i s_i.
// value > 0 proves the primal infeasible (for a feasible x0, r'x0 = d'(A x0) <= the support
// term, so value <= 0). A term whose bound is absent with a nonzero coefficient makes the
// value -inf (not a certificate). Returns value / (sum of |terms|), or -1 (thread 0).
__device__ double b_farkas_ray(const LpView& v, double* scratch);

__device__ double b_farkas(const LpView& v, Ctl* c, double* scratch) {
  const int cur = c->cur;
  for (int i = threadIdx.x; i < v.m; i += blockDim.x) {
    v.ray[i] = (v.y[cur][i] - v.y_rst[i]) * v.dr[i];
  }
  __syncthreads();
  return b_farkas_ray(v, scratch);
}

// The same test of the direction already in v.ray.
__device__ double b_farkas_ray(const LpView& v, double* scratch) {
  const int T = blockDim.x, t = threadIdx.x;
  double acc[3] = {0.0, 0.0, 0.0};  // value, magnitude, absent-bound flags
  for (int i = t; i < v.m; i += T) {
    const double d = v.ray[i];
    const double rl = v.rl[i], ru = v.ru[i];
    if (d > 0.0) {
      if (finite_bound(ru)) {
        acc[0] -= d * ru;
        acc[1] += fabs(d * ru);
      } else {
        acc[2] += 1.0;
      }
    } else if (d < 0.0) {
      if (finite_bound(rl)) {
        acc[0] -= d * rl;
        acc[1] += fabs(d * rl);
      } else {
        acc[2] += 1.0;
      }
    }
  }
  __syncthreads();
  for (int j = t; j < v.n; j += T) {
    double r = 0.0;
    for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) r = fma(v.craw[k], v.ray[v.ci[k]], r);
    const double lj = v.l[j], uj = v.u[j];
    if (r > 0.0) {
      if (finite_bound(lj)) {
        acc[0] += r * lj;
        acc[1] += fabs(r * lj);
      } else {
        acc[2] += 1.0;
      }
    } else if (r < 0.0) {
      if (finite_bound(uj)) {
        acc[0] += r * uj;
        acc[1] += fabs(r * uj);
      } else {
        acc[2] += 1.0;
      }
    }
  }
  double tot[3];
  block_sum<3>(acc, scratch, tot);
  double share = -1.0;
  if (t == 0 && tot[2] == 0.0 && tot[1] > 0.0) share = tot[0] / tot[1];
  return share;
}

// The vector half of the tick decisions (k_eval_apply): best point copy, restart anchors.
__device__ void b_apply(const LpView& v, const Ctl* c) {
  const int T = blockDim.x, t = threadIdx.x;
  const int copy = c->copy_best;
  const bool restart = c->do_restart != 0;
  if (copy == 0 && !restart) return;
  const int cur = c->cur;
  for (int j = t; j < v.n; j += T) {
    if (copy) v.best_x[j] = v.xu[copy - 1][j];
    if (restart) {
      v.x_rst[j] = v.x[cur][j];
      v.x_sum[j] = 0.0;
    }
  }
  for (int i = t; i < v.m; i += T) {
    if (copy) v.best_y[i] = v.yu[copy - 1][i];
    if (restart) {
      v.y_rst[i] = v.y[cur][i];
      v.y_sum[i] = 0.0;
    }
  }
  __syncthreads();
}

// Four blocks per SM: the LP's pointers live in shared memory (s_view), not in registers.
__global__ void __launch_bounds__(kBatchMaxThreads, 2) k_batch_solve(BatchBuffers b) {
  __shared__ double scratch[kBScratch];
  __shared__ int s_item;
  __shared__ Ctl s_ctl;
  __shared__ LpView s_view;
  __shared__ int s_infeasible;
  __shared__ double s_farkas;
  const int T = blockDim.x, t = threadIdx.x;
  Ctl* c = &s_ctl;
  for (int w = next_item(&b.queue[1], b.ninstances, &s_item); w >= 0;
       w = next_item(&b.queue[1], b.ninstances, &s_item)) {
    const int li = b.order[w];
    const BatchInstance I = b.instances[li];
    const BatchMatrix M = b.matrices_out[I.matrix];
    if (t == 0) s_view = make_view(b, I, M);
    __syncthreads();
    const LpView& v = s_view;
    // Scaled problem (src/la/scaling.cpp:124-145), start point and sums (pdhg.cpp:140-190).
    for (int j = t; j < v.n; j += T) {
      const double d = v.dc[j];
      v.cs[j] = v.cost[j] * d;
      const double inv = 1.0 / d;
      const double lj = finite_bound(v.l[j]) ? v.l[j] * inv : -HUGE_VAL;
      const double uj = finite_bound(v.u[j]) ? v.u[j] * inv : HUGE_VAL;
      v.ls[j] = lj;
      v.us[j] = uj;
      const double x0 = clamp_box(0.0, lj, uj);
      v.x[0][j] = x0;
      v.x_rst[j] = x0;
      v.best_x[j] = x0;  // the SCALED start point, as the reference's best_x starts
      v.x_sum[j] = 0.0;
    }
    for (int i = t; i < v.m; i += T) {
      const double d = v.dr[i];
      v.rls[i] = finite_bound(v.rl[i]) ? v.rl[i] * d : -HUGE_VAL;
      v.rus[i] = finite_bound(v.ru[i]) ? v.ru[i] * d : HUGE_VAL;
      v.y[0][i] = 0.0;
      v.y_rst[i] = 0.0;
      v.best_y[i] = 0.0;
      v.y_sum[i] = 0.0;
    }
    {
      unsigned long long* words = reinterpret_cast<unsigned long long*>(c);
      for (int k = t; k < static_cast<int>(sizeof(Ctl) / sizeof(unsigned long long)); k += T) {
        words[k] = 0ull;
      }
    }
    __syncthreads();
    if (t == 0) {
      const double norm = M.spectral_norm;
      c->eta = norm > 0.0 ? 1.0 / norm : 1.0;
      c->omega = 1.0;
      c->spectral_norm = norm;
      c->eta_ceiling = 1.0e3 / dmax(norm, 1e-12);
      c->restart_kkt = HUGE_VAL;
      c->tolerance = b.tolerance;
      c->iteration_limit = b.iteration_limit;
      c->use_restarts = b.use_restarts;
      c->stop_at_request = b.stop_at_request;
      c->stop_rule = b.stop_rule;
      c->best.primal = c->best.dual = c->best.gap = HUGE_VAL;
      c->done = kRunning;
      s_infeasible = 0;
      s_farkas = 0.0;
    }
    __syncthreads();
    int farkas_hits = 0;
    for (;;) {
      if (t == 0) {
        c->eval_now = 0;
        c->copy_best = 0;
        c->do_restart = 0;
        if (c->iteration >= c->iteration_limit) c->done = kIterationLimit;
      }
      __syncthreads();
      if (c->done != kRunning) break;
      b_primal(v, c, scratch);
      b_dual(v, c, scratch);
      if (c->eval_now && c->done == kRunning) {
        b_evaluate(v, c, scratch, false);
        if (b.detect_infeasibility && c->done == kRunning) {
          const double share = b_farkas(v, c, scratch);
          if (t == 0) {
            farkas_hits = share > kFarkasShare ? farkas_hits + 1 : 0;
            if (farkas_hits >= 2) {
              s_infeasible = 1;
              s_farkas = share;
              c->done = kConverged;  // ends the loop; the status says infeasible
            }
          }
          __syncthreads();
        }
        b_apply(v, c);
      }
    }
    // The final evaluation of the reported point (final_mode of the single-LP engine).
    b_evaluate(v, c, scratch, true);
    if (t == 0) {
      BatchOutcome o;
      const Residuals& f = c->final_residuals;
      const bool converged = c->done == kConverged && !s_infeasible;
      const bool verifiable = converged && meets_project_standard(f);
      o.status = s_infeasible ? SANKHYA_GB300_INFEASIBLE
                              : (verifiable ? SANKHYA_GB300_OPTIMAL
                                            : (converged ? SANKHYA_GB300_FEASIBLE
                                                         : SANKHYA_GB300_ITERATION_LIMIT));
      o.converged = converged;
      o.iterations = c->iteration;
      o.attempts = c->attempts;
      o.restarts = c->restarts;
      o.evaluations = c->evaluations;
      o.final_residuals = f;
      o.objective = I.offset + c->model_objective;
      o.dual_bound = verifiable ? I.sense * f.dual_objective + I.offset
                                : (I.sense < 0.0 ? HUGE_VAL : -HUGE_VAL);
      o.farkas_value = s_infeasible ? s_farkas : 0.0;
      o.error = 0;
      b.outcome[li] = o;
    }
  }
}

// ---- Mixed precision, one LP per block ----------------------------------------------------
// The single-LP engine's mixed method (mixed.cuh, Engine::solve_mixed) restated for a block:
// FP32 PDHG on the correction problem u = Dp (x - xbar), v = Dd (y - ybar) around an FP64
// anchor, FP64 step size / primal weight / restart decisions and correction-form KKT
// estimates; a round ends at each inner restart (the anchor moves to the current iterate)
// or when the estimate meets the round's target (the anchor moves to the best candidate),
// and the exact FP64 evaluation of the anchor decides convergence. The anchor lives in the
// FP64 iterate arrays (x[0] = xbar, y[0] = ybar, y[1] = A xbar, x[1] = A' ybar).
struct MixView {
  float *u[2], *u_sum, *u_rst, *cf, *lf, *uf, *uc[2], *u_best;
  float2* ud;
  float *v[2], *v_sum, *v_rst, *gu, *gl, *yhat, *vc[2], *v_best;
  const float *csf, *rsf;
};

__device__ MixView make_mix_view(const BatchBuffers& b, const BatchInstance& I,
                                 const BatchMatrix& M) {
  MixView f;
  const long long c = I.col, r = I.row;
  f.u[0] = b.u0 + c;
  f.u[1] = b.u1 + c;
  f.u_sum = b.u_sum + c;
  f.u_rst = b.u_rst + c;
  f.cf = b.cf + c;
  f.lf = b.lf + c;
  f.uf = b.uf + c;
  f.uc[0] = b.uc0 + c;
  f.uc[1] = b.uc1 + c;
  f.u_best = b.u_best + c;
  f.ud = b.ud + c;
  f.v[0] = b.v0 + r;
  f.v[1] = b.v1 + r;
  f.v_sum = b.v_sum + r;
  f.v_rst = b.v_rst + r;
  f.gu = b.gu + r;
  f.gl = b.gl + r;
  f.yhat = b.yhat + r;
  f.vc[0] = b.vc0 + r;
  f.vc[1] = b.vc1 + r;
  f.v_best = b.v_best + r;
  f.csf = b.csc_f + M.nz;
  f.rsf = b.csr_f + M.nz;
  return f;
}

__device__ bool batch_round_stop(const Ctl* c, const Residuals& r) {
  return worst(r) <= c->round_target;
}

// The FP32 column pass (k_primal_f's arithmetic).
__device__ void bm_primal(const LpView& v, const MixView& f, Ctl* c, double* scratch) {
  const int T = blockDim.x;
  const int cur = c->cur;
  const float* u = f.u[cur];
  float* un = f.u[cur ^ 1];
  const float* vv = f.v[cur];
  const double omega = c->omega;
  const float tau = static_cast<float>(c->eta / omega);
  const bool add = c->pending_add != 0;
  float mvf = 0.0f;
  const int L = v.lanes, G = T / L, sub = threadIdx.x & (L - 1);
  for (int base = 0; base < v.n; base += G) {
    const int j = base + static_cast<int>(threadIdx.x) / L;
    float acc = 0.0f;
    if (j < v.n) {
      for (int k = v.cp[j] + sub; k < v.cp[j + 1]; k += L) acc = fmaf(f.csf[k], vv[v.ci[k]], acc);
    }
    acc = lanes_sum(acc, L);
    if (j >= v.n || sub != 0) continue;
    const float uj = u[j];
    if (add) f.u_sum[j] += uj;
    const float g = f.cf[j] + acc;
    const float unj = clamp_box(fmaf(-tau, g, uj), f.lf[j], f.uf[j]);
    un[j] = unj;
    const float d = unj - uj;
    f.ud[j] = make_float2(fmaf(2.0f, unj, -uj), d);
    mvf = fmaf(d, d, mvf);
  }
  double mv[1] = {static_cast<double>(mvf)}, out[1];
  block_sum<1>(mv, scratch, out);
  if (threadIdx.x == 0) c->mv_primal = 0.5 * omega * out[0];
  __syncthreads();
}

// The FP32 row pass with the correction-form prox (k_dual_f's arithmetic) and the decision.
__device__ void bm_dual(const LpView& v, const MixView& f, Ctl* c, double* scratch) {
  const int T = blockDim.x;
  const int cur = c->cur;
  const float* vv = f.v[cur];
  float* vn = f.v[cur ^ 1];
  const double omega = c->omega;
  const float sigma = static_cast<float>(c->eta * omega);
  const float inv_sigma = 1.0f / sigma;
  const bool add = c->pending_add != 0;
  float a0 = 0.0f, a1 = 0.0f;
  const int L = v.lanes, G = T / L, sub = threadIdx.x & (L - 1);
  for (int base = 0; base < v.m; base += G) {
    const int i = base + static_cast<int>(threadIdx.x) / L;
    float s0 = 0.0f, s1 = 0.0f;
    if (i < v.m) {
      for (int k = v.rp[i] + sub; k < v.rp[i + 1]; k += L) {
        const float2 p = f.ud[v.ri[k]];
        s0 = fmaf(f.rsf[k], p.x, s0);
        s1 = fmaf(f.rsf[k], p.y, s1);
      }
    }
    s0 = lanes_sum(s0, L);
    s1 = lanes_sum(s1, L);
    if (i >= v.m || sub != 0) continue;
    const float vi = vv[i];
    if (add) f.v_sum[i] += vi;
    const float gu = f.gu[i], gl = f.gl[i];
    float vni;
    if (gu == gl) {
      vni = fmaf(sigma, gu + s0, vi);
    } else {
      const float yh = f.yhat[i];
      const float tt = fmaf(yh + vi, inv_sigma, s0);
      if (tt + gu > 0.0f) vni = fmaf(sigma, gu + s0, vi);
      else if (tt + gl < 0.0f) vni = fmaf(sigma, gl + s0, vi);
      else vni = -yh;
    }
    vn[i] = vni;
    const float d = vni - vi;
    a0 = fmaf(d, d, a0);
    a1 = fmaf(d, s1, a1);
  }
  double acc[2] = {static_cast<double>(a0), static_cast<double>(a1)}, tot[2];
  block_sum<2>(acc, scratch, tot);
  if (threadIdx.x == 0 && c->done == kRunning) {
    const double movement = c->mv_primal + (0.5 * tot[0]) / omega;
    step_decision(c, movement, fabs(tot[1]));
  }
  __syncthreads();
}

// The inner evaluation in correction form (k_evalf_rows0 / cols / rows1) and its decisions.
__device__ void bm_evaluate(const LpView& v, const MixView& f, Ctl* c, double* scratch) {
  const int T = blockDim.x, t = threadIdx.x;
  const int cur = c->cur;
  const bool avg = c->averaged > 0;
  const bool pend = c->pending_add != 0;
  const float count = static_cast<float>(c->averaged);
  const int nc = avg ? 2 : 1;
  // s: [0] pviol0 [1] gapr0 [2] pviol1 [3] gapr1 [4] rviol0 [5] rviol1 [6] dv^2
  //    [7] cviol0 [8] gapc0 [9] cviol1 [10] gapc1 [11] du^2 [12] c'u0 [13] c'u1
  double s[14];
#pragma unroll
  for (int q = 0; q < 14; ++q) s[q] = 0.0;
  for (int i = t; i < v.m; i += T) {
    const float vcur = f.v[cur][i];
    float cand[2] = {vcur, 0.0f};
    if (avg) cand[1] = (pend ? f.v_sum[i] + vcur : f.v_sum[i]) / count;
    const float gu = f.gu[i], gl = f.gl[i], yh = f.yhat[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      f.vc[q][i] = cand[q];
      const double yc = static_cast<double>(yh) + static_cast<double>(cand[q]);
      if ((yc > 0.0 && isinf(gu)) || (yc < 0.0 && isinf(gl))) s[4 + q] += yc * yc;
    }
    const double d = static_cast<double>(vcur) - static_cast<double>(f.v_rst[i]);
    s[6] += d * d;
  }
  __syncthreads();
  const int L = v.lanes, G = T / L, sub = t & (L - 1);
  for (int base = 0; base < v.n; base += G) {
    const int j = base + t / L;
    float sq[2] = {0.0f, 0.0f};
    if (j < v.n) {
      for (int k = v.cp[j] + sub; k < v.cp[j + 1]; k += L) {
        const int row = v.ci[k];
        sq[0] = fmaf(f.csf[k], f.vc[0][row], sq[0]);
        if (avg) sq[1] = fmaf(f.csf[k], f.vc[1][row], sq[1]);
      }
    }
    sq[0] = lanes_sum(sq[0], L);
    sq[1] = lanes_sum(sq[1], L);
    if (j >= v.n || sub != 0) continue;
    const float ucur = f.u[cur][j];
    float cand[2] = {ucur, 0.0f};
    if (avg) cand[1] = (pend ? f.u_sum[j] + ucur : f.u_sum[j]) / count;
    const float lf = f.lf[j], uf = f.uf[j], cf = f.cf[j];
    const double cj = v.cs[j];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      f.uc[q][j] = cand[q];
      const double d = static_cast<double>(cf) + static_cast<double>(sq[q]);
      const double uq = static_cast<double>(cand[q]);
      if (d > 0.0) {
        if (isinf(lf)) s[7 + 2 * q] += d * d; else s[8 + 2 * q] += d * (uq - lf);
      } else if (d < 0.0) {
        if (isinf(uf)) s[7 + 2 * q] += d * d; else s[8 + 2 * q] += d * (uq - uf);
      }
      s[12 + q] += cj * uq;
    }
    const double d = static_cast<double>(ucur) - static_cast<double>(f.u_rst[j]);
    s[11] += d * d;
  }
  __syncthreads();
  for (int base = 0; base < v.m; base += G) {
    const int i = base + t / L;
    float a[2] = {0.0f, 0.0f};
    if (i < v.m) {
      for (int k = v.rp[i] + sub; k < v.rp[i + 1]; k += L) {
        const int col = v.ri[k];
        a[0] = fmaf(f.rsf[k], f.uc[0][col], a[0]);
        if (avg) a[1] = fmaf(f.rsf[k], f.uc[1][col], a[1]);
      }
    }
    a[0] = lanes_sum(a[0], L);
    a[1] = lanes_sum(a[1], L);
    if (i >= v.m || sub != 0) continue;
    const double gu = f.gu[i], gl = f.gl[i], yh = f.yhat[i];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= nc) break;
      const double aq = a[q];
      const double eu = gu + aq;
      const double el = -(gl + aq);
      const double viol = dmax(0.0, dmax(eu, el));
      s[2 * q] += viol * viol;
      const double yc = yh + static_cast<double>(f.vc[q][i]);
      if (yc > 0.0 && !isinf(gu)) s[2 * q + 1] += yc * eu;
      else if (yc < 0.0 && !isinf(gl)) s[2 * q + 1] += yc * (gl + aq);
    }
  }
  double tt[14];
  block_sum<14>(s, scratch, tt);
  if (t == 0) {
    const double dp = c->dp, dd = c->dd;
    auto assemble = [&](double pv, double gr, double rv, double cv, double gc, double cu) {
      Residuals r;
      r.absolute_primal = sqrt(pv) / dp;
      r.primal = r.absolute_primal / (1.0 + c->bound_norm_s);
      r.absolute_dual = sqrt(cv + rv) / dd;
      r.dual = r.absolute_dual / (1.0 + c->cost_norm_s);
      const double gap = (gc - gr) / (dp * dd);
      r.primal_objective = c->pobj0 + cu / dp;
      r.dual_objective = r.primal_objective - gap;
      r.gap = fabs(gap) / (1.0 + fabs(r.primal_objective) + fabs(r.dual_objective));
      r.gap_as_verified = fabs(gap) / dmax(1.0, fabs(r.primal_objective));
      r.complementarity = 0.0;
      return r;
    };
    const Residuals rc = assemble(tt[0], tt[1], tt[4], tt[7], tt[8], tt[12]);
    Residuals ra;
    if (avg) ra = assemble(tt[2], tt[3], tt[5], tt[9], tt[10], tt[13]);
    tick_decisions(c, rc, avg ? &ra : nullptr, batch_round_stop, tt[11], tt[6], 1e-10, 1e10);
  }
  __syncthreads();
  // The vector half of the decisions (k_evalf_apply).
  const int copy = c->copy_best;
  const bool restart = c->do_restart != 0;
  if (copy != 0 || restart) {
    const int cc = c->cur;
    for (int j = t; j < v.n; j += T) {
      if (copy) f.u_best[j] = f.uc[copy - 1][j];
      if (restart) {
        f.u_rst[j] = f.u[cc][j];
        f.u_sum[j] = 0.0f;
      }
    }
    for (int i = t; i < v.m; i += T) {
      if (copy) f.v_best[i] = f.vc[copy - 1][i];
      if (restart) {
        f.v_rst[i] = f.v[cc][i];
        f.v_sum[i] = 0.0f;
      }
    }
    __syncthreads();
  }
}

// Four blocks per SM, as k_batch_solve.
__global__ void __launch_bounds__(kBatchMaxThreads, 2) k_batch_solve_mixed(BatchBuffers b) {
  __shared__ double scratch[kBScratch];
  __shared__ int s_item;
  __shared__ Ctl s_ctl;  // the inner loop's control block
  __shared__ Ctl s_fin;  // the exact evaluation's
  __shared__ LpView s_view;
  __shared__ MixView s_mix;
  __shared__ double s_r[8];  // round scalars: [0] dp [1] dd [2] target [3..5] measures
  __shared__ int s_flags[4];  // [0] converged [1] stop [2] infeasible [3] round source
  const int T = blockDim.x, t = threadIdx.x;
  Ctl* c = &s_ctl;
  for (int w = next_item(&b.queue[1], b.ninstances, &s_item); w >= 0;
       w = next_item(&b.queue[1], b.ninstances, &s_item)) {
    const int li = b.order[w];
    const BatchInstance I = b.instances[li];
    const BatchMatrix M = b.matrices_out[I.matrix];
    if (t == 0) {
      s_view = make_view(b, I, M);
      s_mix = make_mix_view(b, I, M);
    }
    __syncthreads();
    const LpView& v = s_view;
    const MixView& f = s_mix;
    // Scaled problem, anchor at the start point, and the scaled problem's norms.
    double nrm[2] = {0.0, 0.0};  // sum b_i^2 (scaled rows), sum c_j^2 (scaled cost)
    for (int j = t; j < v.n; j += T) {
      const double d = v.dc[j];
      v.cs[j] = v.cost[j] * d;
      const double inv = 1.0 / d;
      const double lj = finite_bound(v.l[j]) ? v.l[j] * inv : -HUGE_VAL;
      const double uj = finite_bound(v.u[j]) ? v.u[j] * inv : HUGE_VAL;
      v.ls[j] = lj;
      v.us[j] = uj;
      const double x0 = clamp_box(0.0, lj, uj);
      v.x[0][j] = x0;
      v.best_x[j] = x0;
      nrm[1] += v.cs[j] * v.cs[j];
    }
    for (int i = t; i < v.m; i += T) {
      const double d = v.dr[i];
      const double rl = finite_bound(v.rl[i]) ? v.rl[i] * d : -HUGE_VAL;
      const double ru = finite_bound(v.ru[i]) ? v.ru[i] * d : HUGE_VAL;
      v.rls[i] = rl;
      v.rus[i] = ru;
      v.y[0][i] = 0.0;
      v.best_y[i] = 0.0;
      const double bb = !isinf(rl) ? rl : (!isinf(ru) ? ru : 0.0);
      nrm[0] += bb * bb;
    }
    double nout[2];
    block_sum<2>(nrm, scratch, nout);
    for (Ctl* z : {&s_ctl, &s_fin}) {
      unsigned long long* words = reinterpret_cast<unsigned long long*>(z);
      for (int k = t; k < static_cast<int>(sizeof(Ctl) / sizeof(unsigned long long)); k += T) {
        words[k] = 0ull;
      }
    }
    __syncthreads();
    if (t == 0) {
      const double norm = M.spectral_norm;
      c->eta = norm > 0.0 ? 1.0 / norm : 1.0;
      c->omega = 1.0;
      c->spectral_norm = norm;
      c->eta_ceiling = 1.0e3 / dmax(norm, 1e-12);
      c->restart_kkt = HUGE_VAL;
      c->tolerance = b.tolerance;
      c->iteration_limit = b.iteration_limit;
      c->use_restarts = b.use_restarts;
      c->inner_mode = 1;
      c->bound_norm_s = sqrt(nout[0]);
      c->cost_norm_s = sqrt(nout[1]);
      s_fin.tolerance = b.tolerance;
      s_fin.stop_rule = b.stop_rule;
      s_fin.stop_at_request = b.stop_at_request;
      s_r[0] = 1.0;
      s_r[1] = 1.0;
      s_r[2] = 0.5 * b.tolerance;
      s_flags[0] = s_flags[1] = s_flags[2] = 0;
    }
    __syncthreads();
    long long rounds = 0;
    int farkas_hits = 0;
    for (;; ++rounds) {
      // Anchor measures in FP64 on the scaled problem (k_round_measure).
      for (int i = t; i < v.m; i += T) {
        double acc = 0.0;
        for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) acc = fma(v.rsv[k], v.x[0][v.ri[k]], acc);
        v.y[1][i] = acc;
      }
      for (int j = t; j < v.n; j += T) {
        double acc = 0.0;
        for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) acc = fma(v.csv[k], v.y[0][v.ci[k]], acc);
        v.x[1][j] = acc;
      }
      __syncthreads();
      double mx[2] = {0.0, 0.0}, ob[1] = {0.0};
      for (int i = t; i < v.m; i += T) {
        const double a = v.y[1][i], rl = v.rls[i], ru = v.rus[i], y = v.y[0][i];
        mx[0] = dmax(mx[0], dmax(rl - a, a - ru));
        if (rl != ru) {
          if (y > 0.0 && a < ru) mx[1] = dmax(mx[1], y);
          if (y < 0.0 && a > rl) mx[1] = dmax(mx[1], -y);
        }
      }
      for (int j = t; j < v.n; j += T) {
        const double d = v.cs[j] + v.x[1][j], x = v.x[0][j], l = v.ls[j], u = v.us[j];
        double res;
        if (l == u) res = 0.0;
        else if (x <= l) res = d < 0.0 ? -d : 0.0;
        else if (x >= u) res = d > 0.0 ? d : 0.0;
        else res = fabs(d);
        mx[1] = dmax(mx[1], res);
        ob[0] = fma(v.cs[j], x, ob[0]);
      }
      double m2[2], o1[1];
      block_max<2>(mx, scratch, m2);
      block_sum<1>(ob, scratch, o1);
      if (t == 0) {
        // Scales of this round's correction (Engine::solve_mixed): 1 / residual, at least
        // 1, at most 1e3 times the last and 1e15 overall.
        const double dp = s_r[0], dd = s_r[1];
        const auto scale = [&](double residual, double prev) {
          if (rounds == 0) return 1.0;
          const double want = 1.0 / dmax(residual, 1e-300);
          return dmax(1.0, dmin(dmin(want, prev * 1e3), 1e15));
        };
        const double dpn = scale(m2[0], dp), ddn = scale(m2[1], dd);
        c->omega = dmin(dmax(c->omega * (ddn / dd) / (dpn / dp), 1e-10), 1e10);
        s_r[0] = dpn;
        s_r[1] = ddn;
        c->dp = dpn;
        c->dd = ddn;
        c->pobj0 = o1[0];
        c->round_target = s_r[2];
        c->cur = 0;
        c->averaged = 0;
        c->pending_add = 0;
        c->done = kRunning;
        c->eval_now = c->copy_best = c->do_restart = 0;
        c->best.primal = c->best.dual = c->best.gap = HUGE_VAL;
      }
      __syncthreads();
      // The correction problem (k_round_build) and its zero start.
      {
        const double dp = s_r[0], dd = s_r[1];
        for (int j = t; j < v.n; j += T) {
          const double x = v.x[0][j];
          f.cf[j] = static_cast<float>(dd * (v.cs[j] + v.x[1][j]));
          f.lf[j] = static_cast<float>(dp * (v.ls[j] - x));
          f.uf[j] = static_cast<float>(dp * (v.us[j] - x));
          f.u[0][j] = 0.0f;
          f.u_sum[j] = 0.0f;
          f.u_rst[j] = 0.0f;
          f.u_best[j] = 0.0f;
        }
        for (int i = t; i < v.m; i += T) {
          const double a = v.y[1][i];
          f.gu[i] = static_cast<float>(dp * (a - v.rus[i]));
          f.gl[i] = static_cast<float>(dp * (a - v.rls[i]));
          f.yhat[i] = static_cast<float>(dd * v.y[0][i]);
          f.v[0][i] = 0.0f;
          f.v_sum[i] = 0.0f;
          f.v_rst[i] = 0.0f;
          f.v_best[i] = 0.0f;
        }
      }
      __syncthreads();
      for (;;) {
        if (t == 0) {
          c->eval_now = 0;
          c->copy_best = 0;
          c->do_restart = 0;
          if (c->iteration >= c->iteration_limit) c->done = kIterationLimit;
        }
        __syncthreads();
        if (c->done != kRunning) break;
        bm_primal(v, f, c, scratch);
        bm_dual(v, f, c, scratch);
        if (c->eval_now && c->done == kRunning) bm_evaluate(v, f, c, scratch);
      }
      // Move the anchor: to the current iterate at a restart, else to the best candidate.
      {
        const bool restart = c->done == kRestartRound;
        const int cc = c->cur;
        const float* us = restart ? f.u[cc] : f.u_best;
        const float* vs = restart ? f.v[cc] : f.v_best;
        const double dp = s_r[0], dd = s_r[1];
        for (int j = t; j < v.n; j += T) {
          const double x = clamp_box(v.x[0][j] + static_cast<double>(us[j]) / dp, v.ls[j], v.us[j]);
          v.x[0][j] = x;
          v.best_x[j] = x * v.dc[j];
        }
        for (int i = t; i < v.m; i += T) {
          const double step = static_cast<double>(vs[i]) / dd;
          v.y[0][i] += step;
          v.best_y[i] = v.y[0][i] * v.dr[i];
          v.ray[i] = step * v.dr[i];
        }
      }
      __syncthreads();
      b_evaluate(v, &s_fin, scratch, true);
      if (t == 0) {
        const Residuals& fr = s_fin.final_residuals;
        s_flags[0] = batch_stop_test(&s_fin, fr) ? 1 : 0;
        s_flags[1] = s_flags[0] || c->done == kIterationLimit ||
                     c->iteration >= c->iteration_limit;
        if (!s_flags[1] && c->done == kConverged) s_r[2] *= 0.3;
      }
      __syncthreads();
      if (s_flags[1]) break;
      if (b.detect_infeasibility) {
        const double share = b_farkas_ray(v, scratch);
        if (t == 0) {
          farkas_hits = share > kFarkasShare ? farkas_hits + 1 : 0;
          if (farkas_hits >= 2) s_flags[2] = 1;
        }
        __syncthreads();
        if (s_flags[2]) break;
      }
    }
    if (t == 0) {
      BatchOutcome o;
      const Residuals& fr = s_fin.final_residuals;
      const bool infeasible = s_flags[2] != 0;
      const bool converged = s_flags[0] != 0 && !infeasible;
      const bool verifiable = converged && meets_project_standard(fr);
      o.status = infeasible ? SANKHYA_GB300_INFEASIBLE
                            : (verifiable ? SANKHYA_GB300_OPTIMAL
                                          : (converged ? SANKHYA_GB300_FEASIBLE
                                                       : SANKHYA_GB300_ITERATION_LIMIT));
      o.converged = converged;
      o.iterations = c->iteration;
      o.attempts = c->attempts;
      o.restarts = c->restarts;
      o.evaluations = c->evaluations;
      o.final_residuals = fr;
      o.objective = I.offset + s_fin.model_objective;
      o.dual_bound = verifiable ? I.sense * fr.dual_objective + I.offset
                                : (I.sense < 0.0 ? HUGE_VAL : -HUGE_VAL);
      o.farkas_value = 0.0;
      o.error = 0;
      b.outcome[li] = o;
      if (b.refinements != nullptr) b.refinements[li] = rounds + 1;
    }
  }
}

// ---- The adjoint and the polish: square solves with the basis matrix ----------------------
// At a nondegenerate optimum with basic columns B (strictly inside their bounds), nonbasic
// columns N at a bound and active rows R (equality rows, and inequality rows whose multiplier
// is nonzero), |B| = |R| and the optimum moves, for small changes of the data, along
//     A_RB dx_B = db_R - A_RN dbound_N,    A_RB' dy_R = dc_B,    dx_N = dbound_N,
// (y the row multipliers as reported, so dy*/db = 0 and df*/db_R = y_R, df*/dc = x*,
// df*/dbound_N = d_N, d = c - A'y the reduced costs). For L with upstream gradients g_x, g_y,
// g_f, with p solving A_RB' p = g_x[B] and q solving A_RB q = g_y[R]:
//     dL/dc = g_f x* + q (on B),   dL/db_R = p + g_f y_R,
//     dL/dbound_N = g_x[N] - A_RN' p + g_f d_N,
// and zero for inactive rows and basic columns' bounds. Both kernels work in the batch's
// minimise space (cost sense * c, as src/pdhg/pdhg.cpp:95-111 folds it); the host folds the
// sense into g_y, g_f and dL/dc, so a maximisation LP is differentiated the same way.
//
// The basis matrix is built once per LP in compact form: B and R numbered 0..|B|-1 in index
// order, A_RB stored as a CSR (lines: active rows; entries: basic-column numbers) and as a
// CSC (lines: basic columns; entries: active-row numbers). The solves' products then read no
// masks and gather from vectors of length |B| kept in shared memory. A square solve
// S u = h (S = A_RB or A_RB') runs as iterative refinement around the normal equations of
// the second kind: u += F z with (S F) z = h - S u and F = S', by conjugate gradients with
// the diagonal of S F (the squared lengths of S's lines) as preconditioner. Each pass starts
// from the current u (the polish from the reported point), so it only removes what is left
// of the residual; the passes stop when the true residual ||h - S u|| is below the tolerance
// relative to ||h||.
struct AdjView {
  const double *gx, *gy;
  double gf;
  double *dc, *dl, *du, *drl, *dru;
  double* kw[kAdjVectors];  // compact vectors (|B| entries used)
  int *bcol, *cpos, *rrow, *rpos;
  int *kcp, *kci, *krp, *kri;
  double *kcv, *krv;
  signed char *cs, *rs;
};

__device__ AdjView make_adj_view(const AdjointBuffers& a, const BatchInstance& I, int li) {
  AdjView w;
  const long long c = I.col, r = I.row, z = a.knz[li];
  w.gx = a.gx + c;
  w.gy = a.gy + r;
  w.gf = a.gf[li];
  w.dc = a.dc + c;
  w.dl = a.dl + c;
  w.du = a.du + c;
  w.drl = a.drl + r;
  w.dru = a.dru + r;
  for (int k = 0; k < kAdjVectors; ++k) w.kw[k] = a.kw[k] + r;
  w.bcol = a.bcol + c;
  w.cpos = a.cpos + c;
  w.rrow = a.rrow + r;
  w.rpos = a.rpos + r;
  w.kcp = a.kcp + c + li;
  w.krp = a.krp + r + li;
  w.kci = a.kci + z;
  w.kri = a.kri + z;
  w.kcv = a.kcv + z;
  w.krv = a.krv + z;
  w.cs = a.col_state + c;
  w.rs = a.row_state + r;
  return w;
}

// block_sum with the totals handed to every thread.
template <int NV>
__device__ __forceinline__ void all_sum(double (&v)[NV], double* scratch, double (&out)[NV]) {
  __shared__ double s_all[NV];
  block_sum<NV>(v, scratch, out);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) s_all[q] = out[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) out[q] = s_all[q];
}

// Exclusive prefix sum of one int per thread over the block (blockDim a multiple of 32);
// *total receives the block's sum. Every thread calls it.
__device__ int block_scan(int v, int* total) {
  __shared__ int s_w[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int s = lane < nw ? s_w[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    s_w[lane] = s;
  }
  __syncthreads();
  const int out = x - v + (warp > 0 ? s_w[warp - 1] : 0);
  *total = s_w[nw - 1];
  __syncthreads();
  return out;
}

// Numbers the k < count with on(k) in index order: list[p] = k and pos[k] = p (-1 for the
// others). Returns how many (to every thread).
template <typename On>
__device__ int compact_set(int count, On on, int* list, int* pos) {
  int base = 0;
  for (int start = 0; start < count; start += blockDim.x) {
    const int k = start + threadIdx.x;
    const bool f = k < count && on(k);
    int total = 0;
    const int e = block_scan(f ? 1 : 0, &total);
    if (k < count) {
      pos[k] = f ? base + e : -1;
      if (f) list[base + e] = k;
    }
    base += total;
  }
  __syncthreads();
  return base;
}

// ptr[k] (k < count) holds line k's length on entry and its first entry on exit; ptr[count]
// receives the total.
__device__ void starts_from_lengths(int* ptr, int count) {
  int base = 0;
  for (int start = 0; start < count; start += blockDim.x) {
    const int k = start + threadIdx.x;
    int total = 0;
    const int e = block_scan(k < count ? ptr[k] : 0, &total);
    if (k < count) ptr[k] = base + e;
    base += total;
  }
  if (threadIdx.x == 0) ptr[count] = base;
  __syncthreads();
}

// The active sets of a reported point (best_x, reduced costs, best_y): column states 0 basic,
// 1 at its lower bound (also a fixed column), 2 at its upper; row states 0 inactive, 1 held at
// row_lower, 2 at row_upper (an equality row is active, on the side its multiplier's sign
// names). Strict complementarity decides, so the rule holds at a moderately accurate point:
// a column is nonbasic when its reduced cost is larger than its distance to the bound that
// cost pushes it against (a basic column has a small reduced cost and room on both sides, a
// nonbasic one the reverse), and an inequality row is active when its multiplier is larger
// than its activity's distance to the side the multiplier names. Returns |B| and |R| (all
// threads).
__device__ void b_active_sets(const LpView& v, const AdjView& w, double* scratch, int* nb,
                              int* nr) {
  const int T = blockDim.x, t = threadIdx.x;
  double counts[2] = {0.0, 0.0};
  for (int j = t; j < v.n; j += T) {
    const double d = v.reduced[j], x = v.best_x[j], lj = v.l[j], uj = v.u[j];
    signed char st = 0;
    if (lj == uj) {
      st = 1;
    } else if (d > 0.0 && finite_bound(lj) && d > x - lj) {
      st = 1;
    } else if (d < 0.0 && finite_bound(uj) && -d > uj - x) {
      st = 2;
    }
    w.cs[j] = st;
    if (st == 0) counts[0] += 1.0;
  }
  for (int i = t; i < v.m; i += T) {
    const double y = v.best_y[i];  // the solver's sign: y > 0 holds the row at its upper side
    const double rl = v.rl[i], ru = v.ru[i];
    signed char st = 0;
    if (rl == ru) {
      st = y > 0.0 ? 2 : 1;
    } else {
      double a = 0.0;
      for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) a = fma(v.rraw[k], v.best_x[v.ri[k]], a);
      if (y > 0.0 && finite_bound(ru) && y > ru - a) st = 2;
      else if (y < 0.0 && finite_bound(rl) && -y > a - rl) st = 1;
    }
    w.rs[i] = st;
    if (st != 0) counts[1] += 1.0;
  }
  double cnt[2];
  block_sum<2>(counts, scratch, cnt);
  __shared__ int s_counts[2];
  if (t == 0) {
    s_counts[0] = static_cast<int>(cnt[0]);
    s_counts[1] = static_cast<int>(cnt[1]);
  }
  __syncthreads();
  *nb = s_counts[0];
  *nr = s_counts[1];
  __syncthreads();
}

// The compact basis matrix of the active sets in w.cs / w.rs (see above). Returns |B|, with
// |R| in *nr; the matrix is built only when they are equal.
__device__ int build_basis(const LpView& v, const AdjView& w, int* nr) {
  const int T = blockDim.x, t = threadIdx.x;
  const int nb = compact_set(v.n, [&](int j) { return w.cs[j] == 0; }, w.bcol, w.cpos);
  const int na = compact_set(v.m, [&](int i) { return w.rs[i] != 0; }, w.rrow, w.rpos);
  *nr = na;
  if (nb != na) return nb;
  for (int p = t; p < nb; p += T) {
    const int i = w.rrow[p];
    int len = 0;
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) len += w.cpos[v.ri[k]] >= 0 ? 1 : 0;
    w.krp[p] = len;
    const int j = w.bcol[p];
    len = 0;
    for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) len += w.rpos[v.ci[k]] >= 0 ? 1 : 0;
    w.kcp[p] = len;
  }
  __syncthreads();
  starts_from_lengths(w.krp, nb);
  starts_from_lengths(w.kcp, nb);
  for (int p = t; p < nb; p += T) {
    const int i = w.rrow[p];
    int o = w.krp[p];
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const int c = w.cpos[v.ri[k]];
      if (c >= 0) {
        w.kri[o] = c;
        w.krv[o] = v.rraw[k];
        ++o;
      }
    }
    const int j = w.bcol[p];
    o = w.kcp[p];
    for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) {
      const int r = w.rpos[v.ci[k]];
      if (r >= 0) {
        w.kci[o] = r;
        w.kcv[o] = v.craw[k];
        ++o;
      }
    }
  }
  __syncthreads();
  return nb;
}

// A compact line matrix: line k holds entries ptr[k] .. ptr[k+1]-1 (positions, values).
struct Lines {
  const int *ptr, *idx;
  const double* val;
};

__device__ __forceinline__ double line_dot(const Lines& L, int k, const double* x) {
  double s = 0.0;
  for (int e = L.ptr[k]; e < L.ptr[k + 1]; ++e) s = fma(L.val[e], x[L.idx[e]], s);
  return s;
}

// Conjugate gradients on (S F) z = h from z = 0, preconditioned by diag. p and t are the
// two gathered vectors (shared memory when |B| fits). Stops when ||h - S F z|| (the
// recurrence's residual) is at most tol ||h||. Returns the iterations.
__device__ int pcg_sf(const Lines& S, const Lines& F, int nb, const double* h, double* z,
                      double* r, double* wv, const double* diag, double* p, double* t,
                      double* scratch, int max_it, double tol) {
  const int T = blockDim.x, th = threadIdx.x;
  double a0[2] = {0.0, 0.0};
  for (int k = th; k < nb; k += T) {
    const double rk = h[k], wk = rk / diag[k];
    z[k] = 0.0;
    r[k] = rk;
    wv[k] = wk;
    p[k] = wk;
    a0[0] = fma(rk, rk, a0[0]);
    a0[1] = fma(rk, wk, a0[1]);
  }
  double s0[2];
  all_sum<2>(a0, scratch, s0);
  const double hnorm = sqrt(s0[0]);
  double rw = s0[1], rnorm = hnorm;
  int it = 0;
  while (hnorm > 0.0 && rnorm > tol * hnorm && it < max_it) {
    double a1[1] = {0.0};
    for (int k = th; k < nb; k += T) {
      const double s = line_dot(F, k, p);
      t[k] = s;
      a1[0] = fma(s, s, a1[0]);
    }
    double pkp[1];
    all_sum<1>(a1, scratch, pkp);  // also publishes t
    if (!(pkp[0] > 0.0)) break;
    const double alpha = rw / pkp[0];
    double a2[2] = {0.0, 0.0};
    for (int k = th; k < nb; k += T) {
      const double s = line_dot(S, k, t);
      z[k] = fma(alpha, p[k], z[k]);
      const double rk = fma(-alpha, s, r[k]), wk = rk / diag[k];
      r[k] = rk;
      wv[k] = wk;
      a2[0] = fma(rk, rk, a2[0]);
      a2[1] = fma(rk, wk, a2[1]);
    }
    double s2[2];
    all_sum<2>(a2, scratch, s2);  // every thread is done reading p and t
    rnorm = sqrt(s2[0]);
    const double beta = s2[1] / rw;
    rw = s2[1];
    for (int k = th; k < nb; k += T) p[k] = fma(beta, p[k], wv[k]);
    __syncthreads();
    ++it;
  }
  return it;
}

constexpr int kRefinePasses = 3;
constexpr double kPassReduction = 1e-12;

// S u = h (F = S') by refinement passes around pcg_sf; u holds the starting point on entry
// and the solution on exit, w.kw[2..6] are used as scratch. Returns the conjugate-gradient
// iterations; *rel receives ||h - S u|| / ||h|| at the end (0 when h = 0).
__device__ int solve_square(const Lines& S, const Lines& F, int nb, const double* h, double* u,
                            const AdjView& w, double* p, double* t, double* scratch, int max_it,
                            double tol, double* rel) {
  const int T = blockDim.x, th = threadIdx.x;
  double* const res = w.kw[2];
  double* const z = w.kw[3];
  double* const r = w.kw[4];
  double* const wv = w.kw[5];
  double* const diag = w.kw[6];
  double a0[1] = {0.0};
  for (int k = th; k < nb; k += T) {
    double d = 0.0;
    for (int e = S.ptr[k]; e < S.ptr[k + 1]; ++e) d = fma(S.val[e], S.val[e], d);
    diag[k] = d > 0.0 ? d : 1.0;
    a0[0] = fma(h[k], h[k], a0[0]);
  }
  double hs[1];
  all_sum<1>(a0, scratch, hs);
  const double hnorm = sqrt(hs[0]);
  int its = 0;
  for (int pass = 0;; ++pass) {
    double a1[1] = {0.0};
    for (int k = th; k < nb; k += T) {
      const double rk = h[k] - line_dot(S, k, u);
      res[k] = rk;
      a1[0] = fma(rk, rk, a1[0]);
    }
    double rs[1];
    all_sum<1>(a1, scratch, rs);
    const double rnorm = sqrt(rs[0]);
    *rel = hnorm > 0.0 ? rnorm / hnorm : 0.0;
    if (*rel <= tol || pass == kRefinePasses) break;
    // A pass reduces its own residual to the final target, and by kPassReduction at least:
    // a solve started next to the answer (a polish from the PDHG point, or from a neighbour's
    // vertex, sankhya_gb300_batch_set_point) must still solve its small correction to full
    // accuracy, or two neighbouring solves carry different errors of the correction's size.
    its += pcg_sf(S, F, nb, res, z, r, wv, diag, p, t, scratch, max_it,
                  fmin(tol * hnorm / rnorm, kPassReduction));
    for (int k = th; k < nb; k += T) u[k] += line_dot(F, k, z);
    __syncthreads();
  }
  return its;
}

// The two gathered vectors of a solve: shared memory when |B| fits, else w.kw[7], w.kw[8].
struct Gathered {
  double *p, *t;
};

__device__ Gathered gathered(const AdjointBuffers& a, const AdjView& w, double* s_vec, int nb) {
  if (nb <= a.smem_vec) return Gathered{s_vec, s_vec + a.smem_vec};
  return Gathered{w.kw[7], w.kw[8]};
}

__global__ void __launch_bounds__(kAdjThreads, 2) k_batch_adjoint(BatchBuffers b,
                                                                   AdjointBuffers a) {
  extern __shared__ double s_vec[];
  __shared__ double scratch[kBScratch];
  __shared__ int s_item;
  __shared__ LpView s_view;
  __shared__ AdjView s_adj;
  const int T = blockDim.x, t = threadIdx.x;
  for (int wk = next_item(&b.queue[2], b.ninstances, &s_item); wk >= 0;
       wk = next_item(&b.queue[2], b.ninstances, &s_item)) {
    const int li = b.order[wk];
    const BatchInstance I = b.instances[li];
    const BatchMatrix M = b.matrices_out[I.matrix];
    if (t == 0) {
      s_view = make_view(b, I, M);
      s_adj = make_adj_view(a, I, li);
    }
    __syncthreads();
    const LpView& v = s_view;
    const AdjView& w = s_adj;
    int nb = 0, nr = 0;
    b_active_sets(v, w, scratch, &nb, &nr);
    nb = build_basis(v, w, &nr);
    int it1 = 0, it2 = 0;
    double res1 = 0.0, res2 = 0.0;
    if (nb != nr) {
      for (int j = t; j < v.n; j += T) w.dc[j] = w.dl[j] = w.du[j] = 0.0;
      for (int i = t; i < v.m; i += T) w.drl[i] = w.dru[i] = 0.0;
    } else {
      const Gathered g = gathered(a, w, s_vec, nb);
      const Lines csr{w.krp, w.kri, w.krv}, csc{w.kcp, w.kci, w.kcv};
      double* const h = w.kw[0];
      double* const u = w.kw[1];
      // q: A_RB q = g_y[R] (the reported multipliers are -y and satisfy A_RB' y_R = c_B).
      for (int k = t; k < nb; k += T) {
        h[k] = w.gy[w.rrow[k]];
        u[k] = 0.0;
      }
      __syncthreads();
      it1 = solve_square(csr, csc, nb, h, u, w, g.p, g.t, scratch, a.max_iterations,
                         a.cg_tolerance, &res1);
      for (int j = t; j < v.n; j += T) {
        const int q = w.cpos[j];
        w.dc[j] = fma(w.gf, v.best_x[j], q >= 0 ? u[q] : 0.0);
      }
      __syncthreads();
      // p: A_RB' p = g_x[B].
      for (int k = t; k < nb; k += T) {
        h[k] = w.gx[w.bcol[k]];
        u[k] = 0.0;
      }
      __syncthreads();
      it2 = solve_square(csc, csr, nb, h, u, w, g.p, g.t, scratch, a.max_iterations,
                         a.cg_tolerance, &res2);
      for (int i = t; i < v.m; i += T) {
        const signed char st = w.rs[i];
        const double yrep = -v.best_y[i];  // the reported multiplier
        const double gi = st != 0 ? u[w.rpos[i]] + w.gf * yrep : 0.0;
        w.drl[i] = st == 1 ? gi : 0.0;
        w.dru[i] = st == 2 ? gi : 0.0;
      }
      for (int j = t; j < v.n; j += T) {
        const signed char st = w.cs[j];
        double gj = 0.0;
        if (st != 0) {
          double atp = 0.0;
          for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) {
            const int q = w.rpos[v.ci[k]];
            if (q >= 0) atp = fma(v.craw[k], u[q], atp);
          }
          gj = w.gx[j] - atp + w.gf * v.reduced[j];
        }
        w.dl[j] = st == 1 ? gj : 0.0;
        w.du[j] = st == 2 ? gj : 0.0;
      }
    }
    if (t == 0) {
      AdjointOutcome o;
      o.basic_cols = nb;
      o.active_rows = nr;
      o.iterations[0] = it1;
      o.iterations[1] = it2;
      o.residual[0] = res1;
      o.residual[1] = res2;
      o.status = nb != nr ? 1
                 : (res1 > 100.0 * a.cg_tolerance || res2 > 100.0 * a.cg_tolerance) ? 2
                                                                                    : 0;
      a.outcome[li] = o;
    }
  }
}

// Active-set polish of a batch solve (the PDHG -> basis hand-off): at the reported point's
// active sets, x_B solves A_RB x_B = b_R - A_RN x_N (x_N at its bounds) and the multipliers
// solve A_RB' y_R = c_B (y = 0 off R), both by the square solves above, started from the
// reported point. The polished point replaces the reported one when the optimum is
// nondegenerate (|B| = |R|) and the point is primal and dual feasible within 1e-9
// (relative); the final evaluation then runs on it and the outcome's residuals, objective
// and status are rewritten.
// AdjointOutcome.status: 0 polished, 1 degenerate, 2 a solve did not converge, 4 not a
// converged solve, 5 the polished point failed the feasibility checks.
__global__ void __launch_bounds__(kAdjThreads, 2) k_batch_polish(BatchBuffers b,
                                                                  AdjointBuffers a) {
  extern __shared__ double s_vec[];
  __shared__ double scratch[kBScratch];
  __shared__ int s_item;
  __shared__ LpView s_view;
  __shared__ AdjView s_adj;
  __shared__ Ctl s_ctl;
  const int T = blockDim.x, t = threadIdx.x;
  for (int wk = next_item(&b.queue[3], b.ninstances, &s_item); wk >= 0;
       wk = next_item(&b.queue[3], b.ninstances, &s_item)) {
    const int li = b.order[wk];
    const BatchInstance I = b.instances[li];
    const BatchMatrix M = b.matrices_out[I.matrix];
    if (t == 0) {
      s_view = make_view(b, I, M);
      s_adj = make_adj_view(a, I, li);
    }
    __syncthreads();
    const LpView& v = s_view;
    const AdjView& w = s_adj;
    const BatchOutcome before = b.outcome[li];
    int nb = 0, nr = 0;
    b_active_sets(v, w, scratch, &nb, &nr);
    AdjointOutcome o{};
    const bool solved = before.status == SANKHYA_GB300_OPTIMAL ||
                        before.status == SANKHYA_GB300_FEASIBLE;
    if (solved) nb = build_basis(v, w, &nr);
    o.basic_cols = nb;
    o.active_rows = nr;
    if (nb != nr || !solved) {
      if (t == 0) {
        o.status = !solved ? 4 : 1;
        a.outcome[li] = o;
      }
      continue;
    }
    const Gathered g = gathered(a, w, s_vec, nb);
    const Lines csr{w.krp, w.kri, w.krv}, csc{w.kcp, w.kci, w.kcv};
    double* const h = w.kw[0];
    double* const u = w.kw[1];
    // x_B from b_R - A_RN x_N, starting at the reported x_B.
    for (int k = t; k < nb; k += T) {
      const int i = w.rrow[k];
      double r = w.rs[i] == 1 ? v.rl[i] : v.ru[i];
      for (int e = v.rp[i]; e < v.rp[i + 1]; ++e) {
        const signed char cj = w.cs[v.ri[e]];
        if (cj != 0) r -= v.rraw[e] * (cj == 1 ? v.l[v.ri[e]] : v.u[v.ri[e]]);
      }
      h[k] = r;
      u[k] = v.best_x[w.bcol[k]];
    }
    __syncthreads();
    int it1 = 0, it2 = 0;
    double res1 = 0.0, res2 = 0.0;
    it1 = solve_square(csr, csc, nb, h, u, w, g.p, g.t, scratch, a.max_iterations,
                       a.cg_tolerance, &res1);
    for (int j = t; j < v.n; j += T) {
      const signed char st = w.cs[j];
      v.xu[1][j] = st == 0 ? u[w.cpos[j]] : (st == 1 ? v.l[j] : v.u[j]);
    }
    __syncthreads();
    // y_R from c_B, starting at the reported multipliers (-y in the solver's sign).
    for (int k = t; k < nb; k += T) {
      h[k] = v.cost[w.bcol[k]];
      u[k] = -v.best_y[w.rrow[k]];
    }
    __syncthreads();
    it2 = solve_square(csc, csr, nb, h, u, w, g.p, g.t, scratch, a.max_iterations,
                       a.cg_tolerance, &res2);
    for (int i = t; i < v.m; i += T) {
      const int q = w.rpos[i];
      v.yu[1][i] = q >= 0 ? -u[q] : 0.0;  // the solver's sign
    }
    // The checks: bounds of x_B, signs of the nonbasic reduced costs, inactive rows' sides.
    double bad[1] = {0.0};
    double cmax[1] = {0.0};
    for (int j = t; j < v.n; j += T) cmax[0] = dmax(cmax[0], fabs(v.cost[j]));
    double cm[1];
    block_max<1>(cmax, scratch, cm);
    __shared__ double s_cmax;
    if (t == 0) s_cmax = dmax(1.0, cm[0]);
    __syncthreads();
    for (int j = t; j < v.n; j += T) {
      const signed char st = w.cs[j];
      const double lj = v.l[j], uj = v.u[j];
      double x = v.xu[1][j];
      if (st == 0) {
        const double tol = 1e-9 * dmax(1.0, dmax(fabs(lj), fabs(uj)));
        if ((finite_bound(lj) && x < lj - tol) || (finite_bound(uj) && x > uj + tol)) {
          bad[0] += 1.0;
        }
        x = clamp_box(x, finite_bound(lj) ? lj : -HUGE_VAL, finite_bound(uj) ? uj : HUGE_VAL);
      } else {
        double aty = 0.0;
        for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) {
          aty = fma(v.craw[k], -v.yu[1][v.ci[k]], aty);
        }
        const double d = v.cost[j] - aty;
        const double tol = 1e-9 * s_cmax;
        if (lj != uj && ((st == 1 && d < -tol) || (st == 2 && d > tol))) bad[0] += 1.0;
      }
      v.xu[1][j] = x;
    }
    __syncthreads();
    for (int i = t; i < v.m; i += T) {
      if (w.rs[i] != 0 || v.rl[i] == v.ru[i]) continue;
      double ax = 0.0;
      for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) ax = fma(v.rraw[k], v.xu[1][v.ri[k]], ax);
      const double rl = v.rl[i], ru = v.ru[i];
      const double tol = 1e-9 * dmax(1.0, dmax(finite_bound(rl) ? fabs(rl) : 0.0,
                                               finite_bound(ru) ? fabs(ru) : 0.0));
      if ((finite_bound(rl) && ax < rl - tol) || (finite_bound(ru) && ax > ru + tol)) {
        bad[0] += 1.0;
      }
    }
    double nbad[1];
    block_sum<1>(bad, scratch, nbad);
    __shared__ int s_accept;
    if (t == 0) {
      const bool converged = res1 <= 100.0 * a.cg_tolerance && res2 <= 100.0 * a.cg_tolerance;
      s_accept = converged && nbad[0] == 0.0;
      o.status = !converged ? 2 : (nbad[0] != 0.0 ? 5 : 0);
    }
    __syncthreads();
    if (s_accept) {
      for (int j = t; j < v.n; j += T) v.best_x[j] = v.xu[1][j];
      for (int i = t; i < v.m; i += T) v.best_y[i] = v.yu[1][i];
      {
        unsigned long long* words = reinterpret_cast<unsigned long long*>(&s_ctl);
        for (int k = t; k < static_cast<int>(sizeof(Ctl) / sizeof(unsigned long long)); k += T) {
          words[k] = 0ull;
        }
      }
      __syncthreads();
      b_evaluate(v, &s_ctl, scratch, true);
      if (t == 0) {
        BatchOutcome out = before;
        const Residuals& f = s_ctl.final_residuals;
        const bool verifiable = meets_project_standard(f);
        out.status = verifiable ? SANKHYA_GB300_OPTIMAL : SANKHYA_GB300_FEASIBLE;
        out.final_residuals = f;
        out.objective = I.offset + s_ctl.model_objective;
        out.dual_bound = verifiable ? I.sense * f.dual_objective + I.offset
                                    : (I.sense < 0.0 ? HUGE_VAL : -HUGE_VAL);
        b.outcome[li] = out;
      }
    }
    if (t == 0) {
      o.iterations[0] = it1;
      o.iterations[1] = it2;
      o.residual[0] = res1;
      o.residual[1] = res2;
      a.outcome[li] = o;
    }
    __syncthreads();
  }
}

}  // namespace

namespace {
size_t adjoint_smem_bytes(int smem_vec) {
  return 2 * static_cast<size_t>(smem_vec) * sizeof(double);
}
}  // namespace

void launch_batch_adjoint(const BatchBuffers& b, const AdjointBuffers& a, int grid,
                          cudaStream_t s) {
  const size_t bytes = adjoint_smem_bytes(a.smem_vec);
  // A failure here stays the last error, which the caller's launch check reports.
  cudaFuncSetAttribute(k_batch_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(bytes));
  k_batch_adjoint<<<grid, kAdjThreads, bytes, s>>>(b, a);
}

void launch_batch_polish(const BatchBuffers& b, const AdjointBuffers& a, int grid,
                         cudaStream_t s) {
  const size_t bytes = adjoint_smem_bytes(a.smem_vec);
  // A failure here stays the last error, which the caller's launch check reports.
  cudaFuncSetAttribute(k_batch_polish, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(bytes));
  k_batch_polish<<<grid, kAdjThreads, bytes, s>>>(b, a);
}

int adjoint_blocks_per_sm(int smem_vec) {
  const size_t bytes = adjoint_smem_bytes(smem_vec);
  int per_sm = 1 << 30;
  for (const void* f : {reinterpret_cast<const void*>(k_batch_adjoint),
                        reinterpret_cast<const void*>(k_batch_polish)}) {
    int n = 0;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(bytes)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kAdjThreads, bytes) !=
            cudaSuccess) {
      cudaGetLastError();
      n = 1;
    }
    per_sm = std::min(per_sm, n);
  }
  return per_sm > 0 ? per_sm : 1;
}

int batch_blocks_per_sm(int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_solve, threads, 0) !=
      cudaSuccess) {
    cudaGetLastError();
  }
  return per_sm > 0 ? per_sm : 1;
}

void launch_batch_scaling(const BatchBuffers& b, int grid, cudaStream_t s) {
  k_batch_scale<<<grid, kBatchThreads, 0, s>>>(b);
}

void launch_batch_solve(const BatchBuffers& b, int grid, int threads, cudaStream_t s) {
  k_batch_solve<<<grid, threads, 0, s>>>(b);
}

void launch_batch_solve_mixed(const BatchBuffers& b, int grid, int threads, cudaStream_t s) {
  k_batch_solve_mixed<<<grid, threads, 0, s>>>(b);
}

int batch_mixed_blocks_per_sm(int threads) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_solve_mixed, threads, 0) !=
      cudaSuccess) {
    cudaGetLastError();
  }
  return per_sm > 0 ? per_sm : 1;
}

}  // namespace sgb

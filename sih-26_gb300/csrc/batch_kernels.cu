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

#include "batch.cuh"
#include "common.cuh"
#include "decisions.cuh"
#include "kernels.cuh"
#include "sankhya_gb300.h"

namespace sgb {
namespace {

constexpr int kBScratch = 16 * (kBatchThreads / 32);
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
};

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
  for (int j = threadIdx.x; j < v.n; j += T) {
    double acc = 0.0;
    for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) acc = fma(v.csv[k], y[v.ci[k]], acc);
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
  for (int i = threadIdx.x; i < v.m; i += T) {
    double s0 = 0.0, s1 = 0.0;
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const double2 p = v.xd[v.ri[k]];
      s0 = fma(v.rsv[k], p.x, s0);
      s1 = fma(v.rsv[k], p.y, s1);
    }
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
  for (int j = t; j < v.n; j += T) {
    double sq[2] = {0.0, 0.0};
    for (int k = v.cp[j]; k < v.cp[j + 1]; ++k) {
      const int row = v.ci[k];
      sq[0] = fma(v.craw[k], v.yu[0][row], sq[0]);
      if (avg) sq[1] = fma(v.craw[k], v.yu[1][row], sq[1]);
    }
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
  for (int i = t; i < v.m; i += T) {
    double a[2] = {0.0, 0.0};
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const int col = v.ri[k];
      a[0] = fma(v.rraw[k], v.xu[0][col], a[0]);
      if (avg) a[1] = fma(v.rraw[k], v.xu[1][col], a[1]);
    }
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
__device__ double b_farkas(const LpView& v, Ctl* c, double* scratch) {
  const int T = blockDim.x, t = threadIdx.x;
  const int cur = c->cur;
  double acc[3] = {0.0, 0.0, 0.0};  // value, magnitude, absent-bound flags
  for (int i = t; i < v.m; i += T) {
    const double d = (v.y[cur][i] - v.y_rst[i]) * v.dr[i];
    v.ray[i] = d;
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
__global__ void __launch_bounds__(kBatchThreads, 4) k_batch_solve(BatchBuffers b) {
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

}  // namespace

int batch_blocks_per_sm() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_solve, kBatchThreads, 0);
  return per_sm > 0 ? per_sm : 1;
}

void launch_batch_scaling(const BatchBuffers& b, int grid, cudaStream_t s) {
  k_batch_scale<<<grid, kBatchThreads, 0, s>>>(b);
}

void launch_batch_solve(const BatchBuffers& b, int grid, cudaStream_t s) {
  k_batch_solve<<<grid, kBatchThreads, 0, s>>>(b);
}

}  // namespace sgb

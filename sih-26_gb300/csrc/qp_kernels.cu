// qp_kernels.cu -- kernels of the convex-QP engine (layout and schedule in qp.cuh).
//
// Arithmetic follows src/qp/qp_condat_vu.cpp:257-326 term by term. The element-wise steps
// round as the reference's do; the sums over a row or column accumulate with FMA in a fixed
// order (the entries' order for one lane, then a fixed tree over the lanes and over the chunks
// of a long item), which differs from the reference's sequential sums by a few ulps.
//
// GB300 retires about two FP64 lane operations per clock per SM, and these passes are bound
// by that pipe rather than by HBM: the per-item epilogue costs as much as a dozen entries of
// the sums. So the epilogues are written for few FP64 instructions, each with the reference's
// rounding:
//   - absent bounds are stored as -inf / +inf (the load maps every bound that
//     is_finite_bound calls absent), so the projection is two compares;
//   - the cost and Q are stored times the sense (exact), so the gradient
//     (sense c + sense Qx) + A'y is two additions with the same bits;
//   - 2 x' - x is one FMA (2 x' is exact);
//   - v / sigma is Markstein's correction of the product with the correctly rounded
//     reciprocal (P. Markstein, "Computation of elementary functions on the IBM RISC
//     System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = v (1/sigma), r = v - sigma q
//     exactly by FMA, q + r (1/sigma) rounded once, which is the correctly rounded quotient
//     for operands and results in the normal range (tests/host/qp_division_check.c holds it to
//     IEEE division).
#include "qp.cuh"

#include <algorithm>

namespace sgb {
namespace {

long long g_qp_launches = 0;

// The gradient of the minimisation-space objective, (sense c + sense (Qx)_j) + (A'y)_j, from
// the stored sense c and the sum over sense Q.
__device__ __forceinline__ double qp_gradient(double cmin, double qxmin, double aty) {
  return __dadd_rn(__dadd_rn(cmin, qxmin), aty);
}

// proj_[lo, hi](v) for bounds stored with absent sides as infinities: the reference's project
// (src/qp/qp_condat_vu.cpp:60-64), a NaN left as it is.
__device__ __forceinline__ double box(double v, double lo, double hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

// v / sigma from inv = RN(1 / sigma) (Markstein's correction, see the file header); an exact
// first product or a non-finite residual keeps the product.
__device__ __forceinline__ double divide(double v, double sigma, double inv) {
  const double q = __dmul_rn(v, inv);
  const double r = fma(-q, sigma, v);
  return (r == 0.0 || r != r) ? q : fma(r, inv, q);
}

// A residual into a running maximum held as the bit pattern of a non-negative double (the
// order of such patterns is the order of the values). A NaN is left out, as std::max(a, NaN)
// leaves a in the reference's loops.
__device__ __forceinline__ void max_bits(unsigned long long* slot, double v) {
  if (v > 0.0) atomicMax(slot, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// The skip test of every step and check kernel: nothing once the stopping test held, nothing
// past the iteration limit. Uniform over the grid (ctl changes only between kernels).
__device__ __forceinline__ bool qp_skip(const QpCtl* ctl, int k) {
  const volatile QpCtl* c = ctl;
  return c->done != 0 || c->base + k + 1 > c->limit;
}

// ---- One-lane sums ------------------------------------------------------------------------
// sum over entries [b, e) of values[q] * vec[index[q]], in entry order, FMA-accumulated onto
// acc. Pairs of entries from an even position on are read as one double2 and one int2 (the
// arrays come from cudaMalloc, so an even position is 16- and 8-byte aligned): two memory
// instructions fewer per pair, the same sum in the same order.
__device__ __forceinline__ double seq_dot(const double* values, const int* index,
                                          const double* vec, int b, int e, double acc) {
  int q = b;
  if ((q & 1) && q < e) {
    acc = fma(values[q], vec[index[q]], acc);
    ++q;
  }
  for (; q + 1 < e; q += 2) {
    const double2 vv = *reinterpret_cast<const double2*>(values + q);
    const int2 ii = *reinterpret_cast<const int2*>(index + q);
    acc = fma(vv.x, vec[ii.x], acc);
    acc = fma(vv.y, vec[ii.y], acc);
  }
  if (q < e) acc = fma(values[q], vec[index[q]], acc);
  return acc;
}

// ---- Staged one-lane sums ----------------------------------------------------------------
// A warp's 32 consecutive items own one contiguous slice of each matrix array. The warp copies
// the slice into its part of shared memory with coalesced loads, then each lane sums its own
// item there in entry order: the same sums, in the same order, as the direct one-lane loop.
// A lane with no item (past the end, or a long item of the chunked path) passes an empty
// range. All 32 lanes must call.

__device__ __forceinline__ void stage_slice(const double* values, const int* index, int begin,
                                            int count, double* sv, int* si) {
  const int lane = threadIdx.x & 31;
#pragma unroll 4
  for (int k = lane; k < count; k += 32) {
    sv[k] = __ldg(values + begin + k);
    si[k] = __ldg(index + begin + k);
  }
}

__device__ __forceinline__ double* stage_values() {
  extern __shared__ __align__(16) unsigned char qp_smem[];
  return reinterpret_cast<double*>(qp_smem) + (threadIdx.x >> 5) * kQpStage;
}

__device__ __forceinline__ int* stage_index() {
  extern __shared__ __align__(16) unsigned char qp_smem[];
  return reinterpret_cast<int*>(qp_smem + kQpWarps * kQpStage * sizeof(double)) +
         (threadIdx.x >> 5) * kQpStage;
}

// (A v)_i over row i's entries [b, e) of the CSR.
__device__ __forceinline__ double staged_row_sum(const QpDev& d, const double* v, int i, int b,
                                                 int e) {
  const int lane = threadIdx.x & 31;
  const int r0 = i - lane;
  int wb = 0, we = 0;
  if (r0 < d.m) {
    wb = d.a_rs[r0];
    we = d.a_rs[min(r0 + 32, d.m)];
  }
  double ax = 0.0;
  if (we - wb <= kQpStage) {
    double* sv = stage_values();
    int* si = stage_index();
    stage_slice(d.a_rv, d.a_ci, wb, we - wb, sv, si);
    __syncwarp();
    for (int q = b - wb; q < e - wb; ++q) ax = fma(sv[q], v[si[q]], ax);
  } else {
    for (int q = b; q < e; ++q) ax = fma(d.a_rv[q], v[d.a_ci[q]], ax);
  }
  return ax;
}

// (Q x)_j over row j of Q's entries [qb, qe) and (A'y)_j over column j of A's [ab, ae).
__device__ __forceinline__ void staged_column_sums(const QpDev& d, const double* x, int j, int qb,
                                                   int qe, int ab, int ae, double* qx,
                                                   double* aty) {
  const int lane = threadIdx.x & 31;
  const int c0 = j - lane;
  int qwb = 0, qwe = 0, awb = 0, awe = 0;
  if (c0 < d.n) {
    const int cn = min(c0 + 32, d.n);
    qwb = d.q_rs[c0];
    qwe = d.q_rs[cn];
    awb = d.a_cs[c0];
    awe = d.a_cs[cn];
  }
  const int lq = qwe - qwb, la = awe - awb;
  double sq = 0.0, sa = 0.0;
  if (lq + la <= kQpStage) {
    double* sv = stage_values();
    int* si = stage_index();
    stage_slice(d.q_v, d.q_ci, qwb, lq, sv, si);
    stage_slice(d.a_cv, d.a_ri, awb, la, sv + lq, si + lq);
    __syncwarp();
    for (int q = qb - qwb; q < qe - qwb; ++q) sq = fma(sv[q], x[si[q]], sq);
    for (int a = lq + ab - awb; a < lq + ae - awb; ++a) sa = fma(sv[a], d.y[si[a]], sa);
  } else {
    for (int q = qb; q < qe; ++q) sq = fma(d.q_v[q], x[d.q_ci[q]], sq);
    for (int a = ab; a < ae; ++a) sa = fma(d.a_cv[a], d.y[d.a_ri[a]], sa);
  }
  *qx = sq;
  *aty = sa;
}

// ---- Column pass ------------------------------------------------------------------------

// The epilogue of column j, run by one lane. Returns the check's residual (check form) and the
// objective term c_j x_j + 0.5 x_j (Qx)_j (check and report forms).
template <int MODE>
__device__ __forceinline__ void column_epilogue(const QpDev& d, double tau, int j,
                                                const double* x, double* xn, double qx,
                                                double aty, double* residual, double* obj) {
  const double xj = x[j];
  const double c = d.cost[j];  // sense c; qx is (sense Q x)_j
  if (MODE == kQpStep) {
    const double g = qp_gradient(c, qx, aty);
    const double t = __dsub_rn(xj, __dmul_rn(tau, g));
    const double xnj = box(t, d.col_lower[j], d.col_upper[j]);
    xn[j] = xnj;
    d.xbar[j] = fma(2.0, xnj, -xj);
  } else {
    if (MODE == kQpCheck) {
      const double g = qp_gradient(c, qx, aty);
      const double stepped = box(__dsub_rn(xj, g), d.col_lower[j], d.col_upper[j]);
      *residual = fabs(__dsub_rn(xj, stepped));
    } else {
      // c + Qx = sense (sense c + sense Qx), exactly.
      d.col_dual[j] =
          __dadd_rn(__dmul_rn(d.sense, __dadd_rn(c, qx)), __dmul_rn(d.sense, aty));
    }
    *obj = d.sense * (c * xj + 0.5 * xj * qx);
  }
}

template <int G, int MODE>
__global__ void __launch_bounds__(kQpThreads) k_qp_column(QpDev d, QpCtl* ctl, int k, int src) {
  grid_dependency_wait();
  if (MODE != kQpReport && qp_skip(ctl, k)) return;
  const double tau = ctl->tau;
  const double* x = src ? d.x1 : d.x0;
  double* xn = src ? d.x0 : d.x1;
  const int lane32 = threadIdx.x & 31;
  if (static_cast<int>(blockIdx.x) < d.col_short_blocks) {
    // Short columns: G lanes per column, in column order.
    const int gid = static_cast<int>(blockIdx.x) * kQpThreads + static_cast<int>(threadIdx.x);
    const int j = gid / G, lane = gid % G;
    int qb = 0, qe = 0, ab = 0, ae = 0;
    bool active = j < d.n;
    if (active) {
      qb = d.q_rs[j];
      qe = d.q_rs[j + 1];
      ab = d.a_cs[j];
      ae = d.a_cs[j + 1];
      if ((qe - qb) + (ae - ab) > kQpLongPerLane * G) {  // a long column: the chunk path's
        active = false;
        qb = qe = ab = ae = 0;
      }
    }
    double qx = 0.0, aty = 0.0;
    if (G == 1 && d.stage) {
      staged_column_sums(d, x, j, qb, qe, ab, ae, &qx, &aty);
    } else if (G == 1) {
      qx = seq_dot(d.q_v, d.q_ci, x, qb, qe, 0.0);
      aty = seq_dot(d.a_cv, d.a_ri, d.y, ab, ae, 0.0);
    } else {
      for (int e = qb + lane; e < qe; e += G) qx = fma(d.q_v[e], x[d.q_ci[e]], qx);
      for (int e = ab + lane; e < ae; e += G) aty = fma(d.a_cv[e], d.y[d.a_ri[e]], aty);
      qx = group_sum<G>(qx);
      aty = group_sum<G>(aty);
    }
    double residual = 0.0, obj = 0.0;
    if (active && lane == 0) column_epilogue<MODE>(d, tau, j, x, xn, qx, aty, &residual, &obj);
    if (MODE != kQpStep) {
      __shared__ double scratch[kQpThreads / 32];
      if (MODE == kQpCheck) {
        const double w = warp_max(residual);
        if (lane32 == 0) max_bits(&ctl->dual_bits, w);
      }
      double v[1] = {obj}, total[1];
      block_sum<1>(v, scratch, total);
      if (threadIdx.x == 0) d.obj_part[blockIdx.x] = total[0];
    }
    return;
  }
  // Long columns: one warp per chunk of the column's entries (row j of Q, then column j of
  // A); the last chunk of a column to finish adds the chunks' sums in order and runs its
  // epilogue.
  const int w = (static_cast<int>(blockIdx.x) - d.col_short_blocks) * (kQpThreads / 32) +
                static_cast<int>(threadIdx.x >> 5);
  if (w >= d.ncol_chunks) return;
  const QpChunk ch = d.col_chunks[w];
  const int j = ch.item;
  const int qb = d.q_rs[j], lq = d.q_rs[j + 1] - qb, ab = d.a_cs[j];
  double qx = 0.0, aty = 0.0;
  for (int v = ch.begin + lane32; v < ch.end; v += 32) {
    if (v < lq) {
      qx = fma(d.q_v[qb + v], x[d.q_ci[qb + v]], qx);
    } else {
      const int e = ab + v - lq;
      aty = fma(d.a_cv[e], d.y[d.a_ri[e]], aty);
    }
  }
  qx = warp_sum(qx);
  aty = warp_sum(aty);
  int last = 1;
  if (ch.count > 1) {
    if (lane32 == 0) {
      __stcg(&d.chunk_part[w], make_double2(qx, aty));
      __threadfence();
      last = atomicAdd(&d.col_tickets[ch.slot], 1u) == static_cast<unsigned>(ch.count - 1);
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    if (lane32 == 0) {
      __threadfence();
      qx = aty = 0.0;
      for (int c = ch.first; c < ch.first + ch.count; ++c) {
        const double2 p = __ldcg(&d.chunk_part[c]);
        qx += p.x;
        aty += p.y;
      }
      d.col_tickets[ch.slot] = 0u;
    }
  }
  if (lane32 == 0) {
    double residual = 0.0, obj = 0.0;
    column_epilogue<MODE>(d, tau, j, x, xn, qx, aty, &residual, &obj);
    if (MODE == kQpCheck) max_bits(&ctl->dual_bits, residual);
    if (MODE != kQpStep) d.long_col_obj[ch.slot] = obj;
  }
}

// ---- Row pass ---------------------------------------------------------------------------

template <int MODE>
__device__ __forceinline__ double row_epilogue(const QpDev& d, double sigma, double inv_sigma,
                                               int i, double ax) {
  if (MODE == kQpStep) {
    // y' = v - sigma proj(v / sigma), v = y + sigma (A xbar)_i (src/qp/qp_condat_vu.cpp:270-276).
    const double v = __dadd_rn(d.y[i], __dmul_rn(sigma, ax));
    const double p = box(divide(v, sigma, inv_sigma), d.row_lower[i], d.row_upper[i]);
    d.y[i] = __dsub_rn(v, __dmul_rn(sigma, p));
    return 0.0;
  }
  const double projected = box(ax, d.row_lower[i], d.row_upper[i]);
  return fabs(__dsub_rn(ax, projected));
}

template <int G, int MODE>
__global__ void __launch_bounds__(kQpThreads) k_qp_row(QpDev d, QpCtl* ctl, int k, int src) {
  grid_dependency_wait();
  if (qp_skip(ctl, k)) return;
  const double sigma = ctl->sigma, inv_sigma = ctl->inv_sigma;
  const double* v = MODE == kQpStep ? d.xbar : (src ? d.x1 : d.x0);
  const int lane32 = threadIdx.x & 31;
  if (static_cast<int>(blockIdx.x) < d.row_short_blocks) {
    const int gid = static_cast<int>(blockIdx.x) * kQpThreads + static_cast<int>(threadIdx.x);
    const int i = gid / G, lane = gid % G;
    int b = 0, e = 0;
    bool active = i < d.m;
    if (active) {
      b = d.a_rs[i];
      e = d.a_rs[i + 1];
      if (e - b > kQpLongPerLane * G) {
        active = false;
        b = e = 0;
      }
    }
    double ax = 0.0;
    if (G == 1 && d.stage) {
      ax = staged_row_sum(d, v, i, b, e);
    } else if (G == 1) {
      ax = seq_dot(d.a_rv, d.a_ci, v, b, e, 0.0);
    } else {
      for (int q = b + lane; q < e; q += G) ax = fma(d.a_rv[q], v[d.a_ci[q]], ax);
      ax = group_sum<G>(ax);
    }
    double residual = 0.0;
    if (active && lane == 0) residual = row_epilogue<MODE>(d, sigma, inv_sigma, i, ax);
    if (MODE == kQpCheck) {
      const double w = warp_max(residual);
      if (lane32 == 0) max_bits(&ctl->primal_bits, w);
    }
    return;
  }
  const int w = (static_cast<int>(blockIdx.x) - d.row_short_blocks) * (kQpThreads / 32) +
                static_cast<int>(threadIdx.x >> 5);
  if (w >= d.nrow_chunks) return;
  const QpChunk ch = d.row_chunks[w];
  const int i = ch.item, b = d.a_rs[i];
  double ax = 0.0;
  for (int q = ch.begin + lane32; q < ch.end; q += 32) ax = fma(d.a_rv[b + q], v[d.a_ci[b + q]], ax);
  ax = warp_sum(ax);
  int last = 1;
  if (ch.count > 1) {
    if (lane32 == 0) {
      __stcg(&d.row_chunk_part[w], make_double2(ax, 0.0));
      __threadfence();
      last = atomicAdd(&d.row_tickets[ch.slot], 1u) == static_cast<unsigned>(ch.count - 1);
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    if (lane32 == 0) {
      __threadfence();
      ax = 0.0;
      for (int c = ch.first; c < ch.first + ch.count; ++c) ax += __ldcg(&d.row_chunk_part[c]).x;
      d.row_tickets[ch.slot] = 0u;
    }
  }
  if (lane32 == 0) {
    const double residual = row_epilogue<MODE>(d, sigma, inv_sigma, i, ax);
    if (MODE == kQpCheck) max_bits(&ctl->primal_bits, residual);
  }
}

// ---- Decision -----------------------------------------------------------------------------

// Sum of the objective partials in a fixed order (short-path blocks, then the long columns
// by slot), plus the offset. One block.
__device__ double objective_total(const QpDev& d) {
  __shared__ double scratch[kQpThreads / 32];
  double s = 0.0;
  for (int b = static_cast<int>(threadIdx.x); b < d.col_short_blocks; b += kQpThreads) {
    s += d.obj_part[b];
  }
  double v[1] = {s}, total[1];
  block_sum<1>(v, scratch, total);
  double obj = total[0];
  if (threadIdx.x == 0) {
    for (int q = 0; q < d.nlong_cols; ++q) obj += d.long_col_obj[q];
    obj += d.offset;
  }
  return obj;
}

__global__ void __launch_bounds__(kQpThreads) k_qp_decide(QpDev d, QpCtl* ctl, int k, int p) {
  grid_dependency_wait();
  if (qp_skip(ctl, k)) return;
  const double obj = objective_total(d);
  if (threadIdx.x != 0) return;
  const long long t = ctl->base + k + 1;
  const double pr = __longlong_as_double(static_cast<long long>(ctl->primal_bits));
  const double dr = __longlong_as_double(static_cast<long long>(ctl->dual_bits));
  ctl->primal = pr;
  ctl->dual = dr;
  ctl->objective = obj;
  ctl->checked = t;
  d.hist[p] = QpHist{t, pr, dr, obj};
  ctl->primal_bits = 0ull;
  ctl->dual_bits = 0ull;
  // src/qp/qp_condat_vu.cpp:323-326.
  if (pr <= ctl->tolerance && dr <= ctl->tolerance) {
    ctl->done = 1;
    ctl->iterations = t;
  }
}

__global__ void k_qp_objective(QpDev d, QpCtl* ctl) {
  grid_dependency_wait();
  const double obj = objective_total(d);
  if (threadIdx.x == 0) ctl->objective = obj;
}

__global__ void k_qp_advance(QpCtl* ctl, int graph_iterations) {
  grid_dependency_wait();
  if (ctl->done) return;
  const long long next = ctl->base + graph_iterations;
  ctl->base = next < ctl->limit ? next : ctl->limit;
}

// ---- Setup --------------------------------------------------------------------------------

// G lanes per row, grid-stride over the rows (a long row is walked by its G lanes: the setup
// products run forty times per solve).
template <int G>
__global__ void __launch_bounds__(kQpThreads) k_qp_spmv(int rows, const int* starts,
                                                        const int* index, const double* values,
                                                        const double* v, double* out) {
  const int lane = static_cast<int>(threadIdx.x) % G;
  const int groups = static_cast<int>(gridDim.x) * (kQpThreads / G);
  const int first = (static_cast<int>(blockIdx.x) * kQpThreads + static_cast<int>(threadIdx.x)) / G;
  // Every group runs the same number of rounds, so the lanes of a warp stay together for the
  // shuffles of group_sum.
  const int rounds = (rows + groups - 1) / groups;
  for (int q = 0; q < rounds; ++q) {
    const int r = first + q * groups;
    double s = 0.0;
    if (r < rows) {
      for (int e = starts[r] + lane; e < starts[r + 1]; e += G) s = fma(values[e], v[index[e]], s);
    }
    s = group_sum<G>(s);
    if (r < rows && lane == 0) out[r] = s;
  }
}

__global__ void __launch_bounds__(kQpThreads) k_qp_dot_partial(const double* a, const double* b,
                                                               int n, double* partials) {
  __shared__ double scratch[kQpThreads / 32];
  double s = 0.0;
  for (int i = static_cast<int>(blockIdx.x) * kQpThreads + static_cast<int>(threadIdx.x); i < n;
       i += kQpDotBlocks * kQpThreads) {
    s = fma(a[i], b[i], s);
  }
  double v[1] = {s}, total[1];
  block_sum<1>(v, scratch, total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total[0];
}

__global__ void __launch_bounds__(kQpThreads) k_qp_dot_final(const double* partials, double* out) {
  __shared__ double scratch[kQpThreads / 32];
  double s = 0.0;
  for (int i = static_cast<int>(threadIdx.x); i < kQpDotBlocks; i += kQpThreads) s += partials[i];
  double v[1] = {s}, total[1];
  block_sum<1>(v, scratch, total);
  if (threadIdx.x == 0) *out = total[0];
}

__global__ void k_qp_scale(double* v, int n, const double* norm2) {
  const double norm = sqrt(*norm2);
  for (int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x); i < n;
       i += static_cast<int>(gridDim.x * blockDim.x)) {
    v[i] = __ddiv_rn(v[i], norm);
  }
}

__global__ void k_qp_row_dual(QpDev d, double* row_dual) {
  for (int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x); i < d.m;
       i += static_cast<int>(gridDim.x * blockDim.x)) {
    row_dual[i] = __dmul_rn(-d.sense, d.y[i]);
  }
}

__global__ void k_qp_init(QpDev d) {
  const int stride = static_cast<int>(gridDim.x * blockDim.x);
  for (int j = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x); j < d.n; j += stride) {
    d.x0[j] = box(0.0, d.col_lower[j], d.col_upper[j]);
    d.x1[j] = 0.0;
    d.xbar[j] = 0.0;
  }
  for (int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x); i < d.m; i += stride) {
    d.y[i] = 0.0;
  }
}

int grid_for(int n) { return n <= 0 ? 0 : std::min((n + kQpThreads - 1) / kQpThreads, 4096); }

template <int MODE>
void column_pass(const QpDev& d, QpCtl* ctl, int k, int src, cudaStream_t s) {
  const int grid = d.col_short_blocks + (d.ncol_chunks + 7) / 8;
  if (grid == 0) return;
  const int smem = d.stage ? kQpStageBytes : 0;
  switch (d.col_lanes) {
    case 1: launch_after(k_qp_column<1, MODE>, grid, kQpThreads, smem, s, d, ctl, k, src); break;
    case 2: launch_after(k_qp_column<2, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 4: launch_after(k_qp_column<4, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 8: launch_after(k_qp_column<8, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 16: launch_after(k_qp_column<16, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    default: launch_after(k_qp_column<32, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
  }
  ++g_qp_launches;
}

template <int MODE>
void row_pass(const QpDev& d, QpCtl* ctl, int k, int src, cudaStream_t s) {
  const int grid = d.row_short_blocks + (d.nrow_chunks + 7) / 8;
  if (grid == 0) return;
  const int smem = d.stage ? kQpStageBytes : 0;
  switch (d.row_lanes) {
    case 1: launch_after(k_qp_row<1, MODE>, grid, kQpThreads, smem, s, d, ctl, k, src); break;
    case 2: launch_after(k_qp_row<2, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 4: launch_after(k_qp_row<4, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 8: launch_after(k_qp_row<8, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    case 16: launch_after(k_qp_row<16, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
    default: launch_after(k_qp_row<32, MODE>, grid, kQpThreads, 0, s, d, ctl, k, src); break;
  }
  ++g_qp_launches;
}

}  // namespace

void qp_launch_column_pass(const QpDev& d, QpCtl* ctl, int mode, int k, int src,
                           cudaStream_t s) {
  if (mode == kQpStep) column_pass<kQpStep>(d, ctl, k, src, s);
  else if (mode == kQpCheck) column_pass<kQpCheck>(d, ctl, k, src, s);
  else column_pass<kQpReport>(d, ctl, k, src, s);
  if (mode == kQpReport) {
    launch_after(k_qp_objective, 1, kQpThreads, 0, s, d, ctl);
    ++g_qp_launches;
  }
}

void qp_launch_row_pass(const QpDev& d, QpCtl* ctl, int mode, int k, int src, cudaStream_t s) {
  if (mode == kQpStep) row_pass<kQpStep>(d, ctl, k, src, s);
  else row_pass<kQpCheck>(d, ctl, k, src, s);
}

void qp_launch_decide(const QpDev& d, QpCtl* ctl, int k, int p, cudaStream_t s) {
  launch_after(k_qp_decide, 1, kQpThreads, 0, s, d, ctl, k, p);
  ++g_qp_launches;
}

void qp_launch_advance(QpCtl* ctl, int graph_iterations, cudaStream_t s) {
  launch_after(k_qp_advance, 1, 1, 0, s, ctl, graph_iterations);
  ++g_qp_launches;
}

void qp_launch_spmv(int rows, const int* starts, const int* index, const double* values,
                    const double* v, double* out, int lanes, cudaStream_t s) {
  if (rows <= 0) return;
  const long long threads = static_cast<long long>(rows) * lanes;
  const int grid = static_cast<int>(std::min<long long>((threads + kQpThreads - 1) / kQpThreads, 8192));
  switch (lanes) {
    case 1: k_qp_spmv<1><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
    case 2: k_qp_spmv<2><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
    case 4: k_qp_spmv<4><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
    case 8: k_qp_spmv<8><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
    case 16: k_qp_spmv<16><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
    default: k_qp_spmv<32><<<grid, kQpThreads, 0, s>>>(rows, starts, index, values, v, out); break;
  }
  ++g_qp_launches;
}

void qp_launch_dot(const double* a, const double* b, int n, double* partials, double* out,
                   cudaStream_t s) {
  k_qp_dot_partial<<<kQpDotBlocks, kQpThreads, 0, s>>>(a, b, n, partials);
  k_qp_dot_final<<<1, kQpThreads, 0, s>>>(partials, out);
  g_qp_launches += 2;
}

void qp_launch_scale(double* v, int n, const double* norm2, cudaStream_t s) {
  if (n <= 0) return;
  k_qp_scale<<<grid_for(n), kQpThreads, 0, s>>>(v, n, norm2);
  ++g_qp_launches;
}

void qp_launch_row_dual(const QpDev& d, double* row_dual, cudaStream_t s) {
  if (d.m <= 0) return;
  k_qp_row_dual<<<grid_for(d.m), kQpThreads, 0, s>>>(d, row_dual);
  ++g_qp_launches;
}

void qp_launch_init(const QpDev& d, cudaStream_t s) {
  const int grid = grid_for(std::max(d.m, d.n));
  if (grid == 0) return;
  k_qp_init<<<grid, kQpThreads, 0, s>>>(d);
  ++g_qp_launches;
}

long long qp_kernel_launch_count() { return g_qp_launches; }

cudaError_t qp_configure_kernels() {
  cudaError_t err = cudaSuccess;
  const auto opt = [&](const void* f) {
    const cudaError_t e =
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kQpStageBytes);
    if (err == cudaSuccess) err = e;
  };
  opt(reinterpret_cast<const void*>(k_qp_column<1, kQpStep>));
  opt(reinterpret_cast<const void*>(k_qp_column<1, kQpCheck>));
  opt(reinterpret_cast<const void*>(k_qp_column<1, kQpReport>));
  opt(reinterpret_cast<const void*>(k_qp_row<1, kQpStep>));
  opt(reinterpret_cast<const void*>(k_qp_row<1, kQpCheck>));
  return err;
}

}  // namespace sgb

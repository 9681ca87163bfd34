// batch.cu -- BatchEngine: packs the LPs of a batch into device arrays (one copy per distinct
// matrix) and runs the scaling and solve launches of batch_kernels.cu.
#include "batch_engine.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <random>
#include <tuple>

namespace sgb {

namespace {

bool finite_bound_host(double v) { return !(std::isinf(v) || std::fabs(v) >= 1e30); }

}  // namespace

BatchEngine::BatchEngine(int device) : device_(device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "no CUDA device is available"};
  }
  if (device < 0 || device >= count) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no such device"};
  }
  SGB_CUDA(cudaSetDevice(device));
  SGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SGB_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device));
  SGB_CUDA(cudaEventCreate(&timing_[0]));
  SGB_CUDA(cudaEventCreate(&timing_[1]));
}

BatchEngine::~BatchEngine() {
  cudaSetDevice(device_);
  for (cudaEvent_t e : timing_) {
    if (e != nullptr) cudaEventDestroy(e);
  }
  if (stream_ != nullptr) cudaStreamDestroy(stream_);
}

void BatchEngine::require_loaded() const {
  if (count_ == 0) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no LPs are loaded"};
}

void BatchEngine::load(int count, const sankhya_gb300_lp* lps) {
  Trace trace("batch load");
  if (count <= 0 || lps == nullptr) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "a batch needs at least one LP"};
  }
  for (int k = 0; k < count; ++k) validate_lp(lps[k]);
  SGB_CUDA(cudaSetDevice(device_));
  count_ = 0;
  solved_ = false;
  mats_.clear();
  inst_.clear();

  // Distinct matrices, by identity of the caller's arrays.
  using Key = std::tuple<const int32_t*, const int32_t*, const double*, int, int>;
  std::map<Key, int> seen;
  std::vector<int> first_lp;  // an LP holding each distinct matrix
  std::vector<int> mat_of(static_cast<size_t>(count));
  for (int k = 0; k < count; ++k) {
    const sankhya_gb300_lp& lp = lps[k];
    const Key key{lp.col_starts, lp.row_index, lp.values, lp.rows, lp.cols};
    auto it = seen.find(key);
    if (it == seen.end()) {
      it = seen.emplace(key, static_cast<int>(first_lp.size())).first;
      first_lp.push_back(k);
    }
    mat_of[static_cast<size_t>(k)] = it->second;
  }

  // Matrices: CSC as given, CSR by the counting-sort transpose (src/la/sparse.cpp:271-302).
  std::vector<int> cptr, cidx, rptr, ridx;
  std::vector<double> cval, rval;
  long long nz = 0, cp = 0, rp = 0;
  mat_n_ = mat_m_ = 0;
  for (int lpk : first_lp) {
    const sankhya_gb300_lp& lp = lps[lpk];
    const int m = lp.rows, n = lp.cols;
    const long long nnz = lp.col_starts[n];
    BatchMatrix M{};
    M.m = m;
    M.n = n;
    M.cptr = cp;
    M.rptr = rp;
    M.col = mat_n_;
    M.row = mat_m_;
    M.nz = nz;
    M.nnz = nnz;
    M.spectral_norm = 1.0;
    mats_.push_back(M);
    cptr.insert(cptr.end(), lp.col_starts, lp.col_starts + n + 1);
    cidx.insert(cidx.end(), lp.row_index, lp.row_index + nnz);
    cval.insert(cval.end(), lp.values, lp.values + nnz);
    std::vector<int> r(static_cast<size_t>(m) + 1, 0);
    for (long long k = 0; k < nnz; ++k) ++r[static_cast<size_t>(lp.row_index[k]) + 1];
    for (int i = 0; i < m; ++i) r[i + 1] += r[i];
    std::vector<int> next(r.begin(), r.end() - 1);
    const size_t base = ridx.size();
    ridx.resize(base + static_cast<size_t>(nnz));
    rval.resize(base + static_cast<size_t>(nnz));
    for (int j = 0; j < n; ++j) {
      for (int k = lp.col_starts[j]; k < lp.col_starts[j + 1]; ++k) {
        const int slot = next[lp.row_index[k]]++;
        ridx[base + slot] = j;
        rval[base + slot] = lp.values[k];
      }
    }
    rptr.insert(rptr.end(), r.begin(), r.end());
    nz += nnz;
    cp += n + 1;
    rp += m + 1;
    mat_n_ += n;
    mat_m_ += m;
  }

  // LPs: their vectors, in the minimise-space of src/pdhg/pdhg.cpp:95-111.
  std::vector<double> cost, col_cost, l, u, rl, ru;
  total_n_ = total_m_ = 0;
  for (int k = 0; k < count; ++k) {
    const sankhya_gb300_lp& lp = lps[k];
    const int m = lp.rows, n = lp.cols;
    const double sense = lp.sense < 0.0 ? -1.0 : 1.0;
    BatchInstance I{};
    I.matrix = mat_of[static_cast<size_t>(k)];
    I.m = m;
    I.n = n;
    I.col = total_n_;
    I.row = total_m_;
    I.sense = sense;
    I.offset = lp.objective_offset;
    double cost_sq = 0.0, bound_sq = 0.0;
    for (int j = 0; j < n; ++j) {
      const double c = sense * lp.col_cost[j];
      cost.push_back(c);
      cost_sq += c * c;
    }
    for (int i = 0; i < m; ++i) {
      const double b = finite_bound_host(lp.row_lower[i])
                           ? lp.row_lower[i]
                           : (finite_bound_host(lp.row_upper[i]) ? lp.row_upper[i] : 0.0);
      bound_sq += b * b;
    }
    I.cost_norm = std::sqrt(cost_sq);
    I.bound_norm = std::sqrt(bound_sq);
    col_cost.insert(col_cost.end(), lp.col_cost, lp.col_cost + n);
    l.insert(l.end(), lp.col_lower, lp.col_lower + n);
    u.insert(u.end(), lp.col_upper, lp.col_upper + n);
    rl.insert(rl.end(), lp.row_lower, lp.row_lower + m);
    ru.insert(ru.end(), lp.row_upper, lp.row_upper + m);
    inst_.push_back(I);
    total_n_ += n;
    total_m_ += m;
  }
  // Largest LPs first, so the last blocks to finish hold small ones.
  std::vector<int> order(static_cast<size_t>(count));
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const BatchMatrix& ma = mats_[static_cast<size_t>(inst_[a].matrix)];
    const BatchMatrix& mb = mats_[static_cast<size_t>(inst_[b].matrix)];
    return ma.nnz + ma.m + ma.n > mb.nnz + mb.m + mb.n;
  });

  cudaStream_t s = stream_;
  const size_t N = static_cast<size_t>(std::max(total_n_, 1LL));
  const size_t M = static_cast<size_t>(std::max(total_m_, 1LL));
  d_mats_.upload(mats_.data(), mats_.size(), s);
  d_mats_out_.upload(mats_.data(), mats_.size(), s);
  d_inst_.upload(inst_.data(), inst_.size(), s);
  d_order_.upload(order.data(), order.size(), s);
  order_ = order;
  d_queue_.allocate(4);
  csc_ptr_.upload(cptr.data(), cptr.size(), s);
  csc_idx_.upload(cidx.data(), cidx.size(), s);
  csc_raw_.upload(cval.data(), cval.size(), s);
  csr_ptr_.upload(rptr.data(), rptr.size(), s);
  csr_idx_.upload(ridx.data(), ridx.size(), s);
  csr_raw_.upload(rval.data(), rval.size(), s);
  csc_s_.allocate(std::max<size_t>(cval.size(), 1));
  csr_s_.allocate(std::max<size_t>(rval.size(), 1));
  for (DeviceArray<double>* a : {&dc_, &col_acc_, &power_v_}) {
    a->allocate(static_cast<size_t>(std::max(mat_n_, 1LL)));
  }
  for (DeviceArray<double>* a : {&dr_, &row_acc_, &power_av_}) {
    a->allocate(static_cast<size_t>(std::max(mat_m_, 1LL)));
  }
  cost_.upload(cost.data(), cost.size(), s);
  col_cost_.upload(col_cost.data(), col_cost.size(), s);
  l_.upload(l.data(), l.size(), s);
  u_.upload(u.data(), u.size(), s);
  rl_.upload(rl.data(), rl.size(), s);
  ru_.upload(ru.data(), ru.size(), s);
  for (DeviceArray<double>* a : {&cs_, &ls_, &us_, &x0_, &x1_, &x_sum_, &x_rst_, &xu0_, &xu1_,
                                 &best_x_, &reduced_}) {
    a->allocate(N);
  }
  xd_.allocate(N);
  for (DeviceArray<double>* a : {&rls_, &rus_, &y0_, &y1_, &y_sum_, &y_rst_, &yu0_, &yu1_,
                                 &best_y_, &ray_}) {
    a->allocate(M);
  }
  outcome_.allocate(static_cast<size_t>(count));
  SGB_CUDA(cudaStreamSynchronize(s));
  count_ = count;
}

void BatchEngine::solve(const sankhya_gb300_params& p, sankhya_gb300_batch_item* items,
                        double* device_seconds) {
  Trace trace("batch solve");
  require_loaded();
  if (p.precision != SANKHYA_GB300_FP64 && p.precision != SANKHYA_GB300_MIXED) {
    throw EngineError{SANKHYA_GB300_ERROR_OPTION, "pdhg_precision must be fp64 or mixed"};
  }
  const bool mixed = p.precision == SANKHYA_GB300_MIXED;
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  if (mixed && !mixed_ready_) {
    const size_t N = static_cast<size_t>(std::max(total_n_, 1LL));
    const size_t M = static_cast<size_t>(std::max(total_m_, 1LL));
    long long nz = 0;
    for (const BatchMatrix& mm : mats_) nz += mm.nnz;
    csc_f_.allocate(static_cast<size_t>(std::max(nz, 1LL)));
    csr_f_.allocate(static_cast<size_t>(std::max(nz, 1LL)));
    for (DeviceArray<float>* a : {&u0_, &u1_, &u_sum_, &u_rst_, &cf_, &lf_, &uf_, &uc0_, &uc1_,
                                  &u_best_}) {
      a->allocate(N);
    }
    ud_.allocate(N);
    for (DeviceArray<float>* a : {&v0_, &v1_, &v_sum_, &v_rst_, &gu_, &gl_, &yhat_, &vc0_, &vc1_,
                                  &v_best_}) {
      a->allocate(M);
    }
    refinements_.allocate(static_cast<size_t>(count_));
    mixed_ready_ = true;
  }
  // The power iteration's start vectors: the reference's std::mt19937(seed + 1) stream with
  // uniform_real_distribution(-1, 1) (src/la/scaling.cpp:168-170), one per matrix.
  std::vector<double> v0(static_cast<size_t>(std::max(mat_n_, 1LL)));
  for (const BatchMatrix& M : mats_) {
    std::mt19937 rng(static_cast<unsigned>(p.random_seed) + 1u);
    std::uniform_real_distribution<double> spread(-1.0, 1.0);
    for (int j = 0; j < M.n; ++j) v0[static_cast<size_t>(M.col + j)] = spread(rng);
  }
  if (mat_n_ > 0) {
    SGB_CUDA(cudaMemcpyAsync(power_v_.ptr, v0.data(), static_cast<size_t>(mat_n_) * sizeof(double),
                             cudaMemcpyHostToDevice, s));
  }
  SGB_CUDA(cudaMemsetAsync(d_queue_.ptr, 0, 4 * sizeof(unsigned int), s));

  BatchBuffers b{};
  b.nmatrices = static_cast<int>(mats_.size());
  b.ninstances = count_;
  b.matrices = d_mats_.ptr;
  b.matrices_out = d_mats_out_.ptr;
  b.instances = d_inst_.ptr;
  b.order = d_order_.ptr;
  b.queue = d_queue_.ptr;
  b.csc_ptr = csc_ptr_.ptr;
  b.csc_idx = csc_idx_.ptr;
  b.csr_ptr = csr_ptr_.ptr;
  b.csr_idx = csr_idx_.ptr;
  b.csc_raw = csc_raw_.ptr;
  b.csr_raw = csr_raw_.ptr;
  b.csc_s = csc_s_.ptr;
  b.csr_s = csr_s_.ptr;
  b.dr = dr_.ptr;
  b.dc = dc_.ptr;
  b.row_acc = row_acc_.ptr;
  b.col_acc = col_acc_.ptr;
  b.power_v = power_v_.ptr;
  b.power_av = power_av_.ptr;
  b.cost = cost_.ptr;
  b.col_cost = col_cost_.ptr;
  b.l = l_.ptr;
  b.u = u_.ptr;
  b.rl = rl_.ptr;
  b.ru = ru_.ptr;
  b.cs = cs_.ptr;
  b.ls = ls_.ptr;
  b.us = us_.ptr;
  b.rls = rls_.ptr;
  b.rus = rus_.ptr;
  b.x0 = x0_.ptr;
  b.x1 = x1_.ptr;
  b.x_sum = x_sum_.ptr;
  b.x_rst = x_rst_.ptr;
  b.xu0 = xu0_.ptr;
  b.xu1 = xu1_.ptr;
  b.best_x = best_x_.ptr;
  b.reduced = reduced_.ptr;
  b.xd = xd_.ptr;
  b.y0 = y0_.ptr;
  b.y1 = y1_.ptr;
  b.y_sum = y_sum_.ptr;
  b.y_rst = y_rst_.ptr;
  b.yu0 = yu0_.ptr;
  b.yu1 = yu1_.ptr;
  b.best_y = best_y_.ptr;
  b.ray = ray_.ptr;
  b.outcome = outcome_.ptr;
  b.tolerance = p.tolerance;
  b.iteration_limit = p.iteration_limit < 0 ? 1000000 : p.iteration_limit;
  b.use_restarts = p.restart != 0;
  b.stop_at_request = p.stop_at_request != 0;
  b.stop_rule = p.stop_rule == SANKHYA_GB300_STOP_RELATIVE ? 1 : 0;
  b.detect_infeasibility = 1;
  b.lanes = 1;
  if (mixed) {
    b.csc_f = csc_f_.ptr;
    b.csr_f = csr_f_.ptr;
    b.u0 = u0_.ptr;
    b.u1 = u1_.ptr;
    b.u_sum = u_sum_.ptr;
    b.u_rst = u_rst_.ptr;
    b.cf = cf_.ptr;
    b.lf = lf_.ptr;
    b.uf = uf_.ptr;
    b.uc0 = uc0_.ptr;
    b.uc1 = uc1_.ptr;
    b.u_best = u_best_.ptr;
    b.ud = ud_.ptr;
    b.v0 = v0_.ptr;
    b.v1 = v1_.ptr;
    b.v_sum = v_sum_.ptr;
    b.v_rst = v_rst_.ptr;
    b.gu = gu_.ptr;
    b.gl = gl_.ptr;
    b.yhat = yhat_.ptr;
    b.vc0 = vc0_.ptr;
    b.vc1 = vc1_.ptr;
    b.v_best = v_best_.ptr;
    b.refinements = refinements_.ptr;
  }

  // The scaling launch runs once; with no schedule set, the candidate schedules are timed on
  // a sample of the batch before the solve (not part of the solve's device time).
  const int scale_grid = std::max(1, std::min(b.nmatrices, num_sms_ * 8));
  SGB_CUDA(cudaEventRecord(timing_[0], s));
  launch_batch_scaling(b, scale_grid, s);
  SGB_CUDA(cudaGetLastError());
  SGB_CUDA(cudaEventRecord(timing_[1], s));
  SGB_CUDA(cudaEventSynchronize(timing_[1]));
  float scale_ms = 0.0f;
  SGB_CUDA(cudaEventElapsedTime(&scale_ms, timing_[0], timing_[1]));
  int lanes = sched_lanes_, threads = sched_threads_;
  last_tune_seconds_ = 0.0;
  if (lanes == 0 || threads == 0) {
    const auto t0 = std::chrono::steady_clock::now();
    autotune(b, mixed, &lanes, &threads);
    last_tune_seconds_ =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  b.lanes = lanes;
  last_lanes_ = lanes;
  last_threads_ = threads;
  buffers_ = b;
  SGB_CUDA(cudaMemsetAsync(d_queue_.ptr, 0, 4 * sizeof(unsigned int), s));
  SGB_CUDA(cudaEventRecord(timing_[0], s));
  if (mixed) {
    const int grid = std::max(1, std::min(count_, num_sms_ * batch_mixed_blocks_per_sm(threads)));
    launch_batch_solve_mixed(b, grid, threads, s);
  } else {
    const int grid = std::max(1, std::min(count_, num_sms_ * batch_blocks_per_sm(threads)));
    launch_batch_solve(b, grid, threads, s);
  }
  SGB_CUDA(cudaGetLastError());
  SGB_CUDA(cudaEventRecord(timing_[1], s));
  std::vector<BatchOutcome> out(static_cast<size_t>(count_));
  std::vector<BatchMatrix> mats(mats_.size());
  std::vector<long long> rounds(static_cast<size_t>(count_), 0);
  if (mixed) {
    SGB_CUDA(cudaMemcpyAsync(rounds.data(), refinements_.ptr, rounds.size() * sizeof(long long),
                             cudaMemcpyDeviceToHost, s));
  }
  SGB_CUDA(cudaMemcpyAsync(out.data(), outcome_.ptr, out.size() * sizeof(BatchOutcome),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(mats.data(), d_mats_out_.ptr, mats.size() * sizeof(BatchMatrix),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  float ms = 0.0f;
  SGB_CUDA(cudaEventElapsedTime(&ms, timing_[0], timing_[1]));
  if (device_seconds != nullptr) *device_seconds = 1e-3 * (scale_ms + ms);
  for (int k = 0; k < count_; ++k) {
    const BatchOutcome& o = out[static_cast<size_t>(k)];
    sankhya_gb300_batch_item& it = items[k];
    it.status = o.status;
    it.converged = o.converged;
    it.iterations = o.iterations;
    it.attempts = o.attempts;
    it.restarts = o.restarts;
    it.evaluations = o.evaluations;
    it.objective = o.objective;
    it.dual_bound = o.dual_bound;
    const Residuals& f = o.final_residuals;
    it.final_residuals = sankhya_gb300_residuals{f.primal,          f.dual,           f.gap,
                                                 f.primal_objective, f.dual_objective,
                                                 f.absolute_primal,  f.absolute_dual,
                                                 f.gap_as_verified,  f.complementarity};
    it.spectral_norm = mats[static_cast<size_t>(inst_[static_cast<size_t>(k)].matrix)].spectral_norm;
    it.farkas_value = o.farkas_value;
    it.refinements = rounds[static_cast<size_t>(k)];
  }
  solved_ = true;
}

void BatchEngine::set_schedule(int lanes, int threads) {
  const bool automatic = lanes == 0 && threads == 0;
  const bool lanes_ok = lanes >= 1 && lanes <= 32 && (lanes & (lanes - 1)) == 0;
  const bool threads_ok = threads == 128 || threads == 256 || threads == 512;
  if (!automatic && !(lanes_ok && threads_ok)) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT,
                      "a batch schedule is lanes 1, 2, 4, 8, 16 or 32 and threads 128, 256 or "
                      "512 (or 0 and 0 to autotune)"};
  }
  sched_lanes_ = lanes;
  sched_threads_ = threads;
}

void BatchEngine::last_schedule(int* lanes, int* threads, double* tune_seconds) const {
  if (lanes != nullptr) *lanes = last_lanes_;
  if (threads != nullptr) *threads = last_threads_;
  if (tune_seconds != nullptr) *tune_seconds = last_tune_seconds_;
}

// The autotuner. Candidates: 1, 2, 4 or 8 lanes per row or column, 128, 256 or 512 threads
// per LP. Each runs the batch's own solve kernel, for kTuneSteps accepted steps, on the same
// sample: up to four LPs per SM taken at even strides through the solve order (so large and
// small LPs are both in it), from scratch, with the batch's own options. The fastest by
// device time wins; the sample's outcomes are overwritten by the solve that follows.
void BatchEngine::autotune(BatchBuffers b, bool mixed, int* lanes, int* threads) {
  constexpr long long kTuneSteps = 200;
  cudaStream_t s = stream_;
  const int sample = std::max(1, std::min(count_, 4 * num_sms_));
  std::vector<int> pick(static_cast<size_t>(sample));
  for (int k = 0; k < sample; ++k) {
    pick[static_cast<size_t>(k)] =
        order_[static_cast<size_t>(static_cast<long long>(k) * count_ / sample)];
  }
  d_tune_order_.upload(pick.data(), pick.size(), s);
  b.order = d_tune_order_.ptr;
  b.ninstances = sample;
  b.iteration_limit = std::min(b.iteration_limit, kTuneSteps);
  float best_ms = 0.0f;
  *lanes = 1;
  *threads = kBatchThreads;
  bool first = true;
  for (int t : {128, 256, 512}) {
    for (int l : {1, 2, 4, 8}) {
      b.lanes = l;
      SGB_CUDA(cudaMemsetAsync(d_queue_.ptr, 0, 4 * sizeof(unsigned int), s));
      SGB_CUDA(cudaEventRecord(timing_[0], s));
      if (mixed) {
        const int grid = std::max(1, std::min(sample, num_sms_ * batch_mixed_blocks_per_sm(t)));
        launch_batch_solve_mixed(b, grid, t, s);
      } else {
        const int grid = std::max(1, std::min(sample, num_sms_ * batch_blocks_per_sm(t)));
        launch_batch_solve(b, grid, t, s);
      }
      SGB_CUDA(cudaGetLastError());
      SGB_CUDA(cudaEventRecord(timing_[1], s));
      SGB_CUDA(cudaEventSynchronize(timing_[1]));
      float ms = 0.0f;
      SGB_CUDA(cudaEventElapsedTime(&ms, timing_[0], timing_[1]));
      if (first || ms < best_ms) {
        best_ms = ms;
        *lanes = l;
        *threads = t;
        first = false;
      }
    }
  }
}

void BatchEngine::solution(int index, double* col_value, double* col_dual, double* row_dual) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  if (index < 0 || index >= count_) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no such LP in the batch"};
  }
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  const BatchInstance& I = inst_[static_cast<size_t>(index)];
  const size_t n = static_cast<size_t>(I.n), m = static_cast<size_t>(I.m);
  std::vector<double> red(n), by(m);
  if (col_value && n > 0) {
    SGB_CUDA(cudaMemcpyAsync(col_value, best_x_.ptr + I.col, n * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  }
  if (n > 0) {
    SGB_CUDA(cudaMemcpyAsync(red.data(), reduced_.ptr + I.col, n * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  }
  if (m > 0) {
    SGB_CUDA(cudaMemcpyAsync(by.data(), best_y_.ptr + I.row, m * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  }
  SGB_CUDA(cudaStreamSynchronize(s));
  if (col_dual) {
    for (size_t j = 0; j < n; ++j) col_dual[j] = I.sense * red[j];
  }
  if (row_dual) {
    for (size_t i = 0; i < m; ++i) row_dual[i] = I.sense * (-by[i]);
  }
}

void BatchEngine::ray(int index, double* ray) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  if (index < 0 || index >= count_) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no such LP in the batch"};
  }
  if (ray == nullptr) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "null ray"};
  SGB_CUDA(cudaSetDevice(device_));
  const BatchInstance& I = inst_[static_cast<size_t>(index)];
  if (I.m > 0) {
    SGB_CUDA(cudaMemcpyAsync(ray, ray_.ptr + I.row, static_cast<size_t>(I.m) * sizeof(double),
                             cudaMemcpyDeviceToHost, stream_));
  }
  SGB_CUDA(cudaStreamSynchronize(stream_));
}

void BatchEngine::set_point(int index, const double* col_value, const double* col_dual,
                            const double* row_dual) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  if (index < 0 || index >= count_) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no such LP in the batch"};
  }
  const BatchInstance& I = inst_[static_cast<size_t>(index)];
  const size_t n = static_cast<size_t>(I.n), m = static_cast<size_t>(I.m);
  if ((n > 0 && (col_value == nullptr || col_dual == nullptr)) || (m > 0 && row_dual == nullptr)) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "null point"};
  }
  SGB_CUDA(cudaSetDevice(device_));
  // The inverse of solution(): col_dual = sense * reduced, row_dual = sense * (-y).
  std::vector<double> red(n), by(m);
  for (size_t j = 0; j < n; ++j) red[j] = I.sense * col_dual[j];
  for (size_t i = 0; i < m; ++i) by[i] = -I.sense * row_dual[i];
  if (n > 0) {
    SGB_CUDA(cudaMemcpyAsync(best_x_.ptr + I.col, col_value, n * sizeof(double),
                             cudaMemcpyHostToDevice, stream_));
    SGB_CUDA(cudaMemcpyAsync(reduced_.ptr + I.col, red.data(), n * sizeof(double),
                             cudaMemcpyHostToDevice, stream_));
  }
  if (m > 0) {
    SGB_CUDA(cudaMemcpyAsync(best_y_.ptr + I.row, by.data(), m * sizeof(double),
                             cudaMemcpyHostToDevice, stream_));
  }
  SGB_CUDA(cudaStreamSynchronize(stream_));
}

void BatchEngine::adjoint(const double* const* dl_dx, const double* const* dl_dy,
                          const double* dl_df, double* const* dl_dc, double* const* dl_drl,
                          double* const* dl_dru, double* const* dl_dl, double* const* dl_du,
                          sankhya_gb300_adjoint_info* info) {
  Trace trace("batch adjoint");
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  const size_t N = static_cast<size_t>(std::max(total_n_, 1LL));
  const size_t M = static_cast<size_t>(std::max(total_m_, 1LL));
  ensure_adjoint_buffers();
  // Upstream gradients, packed in the LPs' vector order.
  std::vector<double> gx(N, 0.0), gy(M, 0.0), gf(static_cast<size_t>(count_), 0.0);
  for (int k = 0; k < count_; ++k) {
    const BatchInstance& I = inst_[static_cast<size_t>(k)];
    if (dl_dx != nullptr && dl_dx[k] != nullptr) {
      std::copy(dl_dx[k], dl_dx[k] + I.n, gx.begin() + I.col);
    }
    // The kernel differentiates the minimise-space LP (cost sense * c, multipliers
    // sense * y): y and f enter with the sense, dL/dc leaves with it (finish_adjoint).
    if (dl_dy != nullptr && dl_dy[k] != nullptr) {
      for (int i = 0; i < I.m; ++i) gy[static_cast<size_t>(I.row + i)] = I.sense * dl_dy[k][i];
    }
    if (dl_df != nullptr) gf[static_cast<size_t>(k)] = I.sense * dl_df[k];
  }
  SGB_CUDA(cudaMemcpyAsync(a_gx_.ptr, gx.data(), N * sizeof(double), cudaMemcpyHostToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(a_gy_.ptr, gy.data(), M * sizeof(double), cudaMemcpyHostToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(a_gf_.ptr, gf.data(), gf.size() * sizeof(double),
                           cudaMemcpyHostToDevice, s));
  AdjointBuffers a = adjoint_buffers();
  SGB_CUDA(cudaMemsetAsync(d_queue_.ptr + 2, 0, sizeof(unsigned int), s));
  const int grid =
      std::max(1, std::min(count_, num_sms_ * adjoint_blocks_per_sm(a.smem_vec)));
  launch_batch_adjoint(buffers_, a, grid, s);
  SGB_CUDA(cudaGetLastError());
  finish_adjoint(dl_dc, dl_drl, dl_dru, dl_dl, dl_du, info);
}

void BatchEngine::ensure_adjoint_buffers() {
  if (adjoint_ready_) return;
  const size_t N = static_cast<size_t>(std::max(total_n_, 1LL));
  const size_t M = static_cast<size_t>(std::max(total_m_, 1LL));
  for (DeviceArray<double>* a : {&a_gx_, &a_dc_, &a_dl_, &a_du_}) a->allocate(N);
  for (DeviceArray<double>* a : {&a_gy_, &a_drl_, &a_dru_}) a->allocate(M);
  for (auto& a : a_kw_) a.allocate(M);
  a_bcol_.allocate(N);
  a_cpos_.allocate(N);
  a_rrow_.allocate(M);
  a_rpos_.allocate(M);
  a_kcp_.allocate(N + static_cast<size_t>(count_));
  a_krp_.allocate(M + static_cast<size_t>(count_));
  // Each LP's compact basis matrix holds at most its matrix's entries.
  std::vector<long long> knz(static_cast<size_t>(count_));
  long long nz = 0;
  int dim = 1;
  for (int k = 0; k < count_; ++k) {
    const BatchInstance& I = inst_[static_cast<size_t>(k)];
    knz[static_cast<size_t>(k)] = nz;
    nz += mats_[static_cast<size_t>(I.matrix)].nnz;
    dim = std::max(dim, std::min(I.m, I.n));
  }
  const size_t Z = static_cast<size_t>(std::max(nz, 1LL));
  a_kci_.allocate(Z);
  a_kri_.allocate(Z);
  a_kcv_.allocate(Z);
  a_krv_.allocate(Z);
  a_knz_.allocate(knz.size());
  SGB_CUDA(cudaMemcpy(a_knz_.ptr, knz.data(), knz.size() * sizeof(long long),
                      cudaMemcpyHostToDevice));
  a_smem_vec_ = std::min(dim, kAdjSmemVec);
  a_gf_.allocate(static_cast<size_t>(count_));
  a_cs_.allocate(N);
  a_rs_.allocate(M);
  a_out_.allocate(static_cast<size_t>(count_));
  adjoint_ready_ = true;
}

AdjointBuffers BatchEngine::adjoint_buffers() {
  AdjointBuffers a{};
  a.gx = a_gx_.ptr;
  a.gy = a_gy_.ptr;
  a.gf = a_gf_.ptr;
  a.dc = a_dc_.ptr;
  a.dl = a_dl_.ptr;
  a.du = a_du_.ptr;
  a.drl = a_drl_.ptr;
  a.dru = a_dru_.ptr;
  for (int k = 0; k < kAdjVectors; ++k) a.kw[k] = a_kw_[k].ptr;
  a.bcol = a_bcol_.ptr;
  a.cpos = a_cpos_.ptr;
  a.rrow = a_rrow_.ptr;
  a.rpos = a_rpos_.ptr;
  a.kcp = a_kcp_.ptr;
  a.krp = a_krp_.ptr;
  a.kci = a_kci_.ptr;
  a.kri = a_kri_.ptr;
  a.kcv = a_kcv_.ptr;
  a.krv = a_krv_.ptr;
  a.knz = a_knz_.ptr;
  a.col_state = a_cs_.ptr;
  a.row_state = a_rs_.ptr;
  a.outcome = a_out_.ptr;
  a.max_iterations = 20000;
  a.cg_tolerance = 1e-13;
  a.smem_vec = a_smem_vec_;
  return a;
}

void BatchEngine::finish_adjoint(double* const* dl_dc, double* const* dl_drl,
                                 double* const* dl_dru, double* const* dl_dl,
                                 double* const* dl_du, sankhya_gb300_adjoint_info* info) {
  cudaStream_t s = stream_;
  const size_t N = static_cast<size_t>(std::max(total_n_, 1LL));
  const size_t M = static_cast<size_t>(std::max(total_m_, 1LL));
  std::vector<double> dc(N), dl(N), du(N), drl(M), dru(M);
  std::vector<AdjointOutcome> out(static_cast<size_t>(count_));
  SGB_CUDA(cudaMemcpyAsync(dc.data(), a_dc_.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(dl.data(), a_dl_.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(du.data(), a_du_.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(drl.data(), a_drl_.ptr, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(dru.data(), a_dru_.ptr, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(out.data(), a_out_.ptr, out.size() * sizeof(AdjointOutcome),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  const auto put = [](double* const* dst, int k, const std::vector<double>& src, long long off,
                      int len) {
    if (dst != nullptr && dst[k] != nullptr) {
      std::copy(src.begin() + off, src.begin() + off + len, dst[k]);
    }
  };
  for (int k = 0; k < count_; ++k) {
    const BatchInstance& I = inst_[static_cast<size_t>(k)];
    if (I.sense < 0.0) {
      for (long long j = I.col; j < I.col + I.n; ++j) {
        dc[static_cast<size_t>(j)] = -dc[static_cast<size_t>(j)];
      }
    }
    put(dl_dc, k, dc, I.col, I.n);
    put(dl_dl, k, dl, I.col, I.n);
    put(dl_du, k, du, I.col, I.n);
    put(dl_drl, k, drl, I.row, I.m);
    put(dl_dru, k, dru, I.row, I.m);
    if (info != nullptr) {
      const AdjointOutcome& o = out[static_cast<size_t>(k)];
      info[k].status = o.status;
      info[k].basic_cols = o.basic_cols;
      info[k].active_rows = o.active_rows;
      info[k].iterations[0] = o.iterations[0];
      info[k].iterations[1] = o.iterations[1];
      info[k].residual[0] = o.residual[0];
      info[k].residual[1] = o.residual[1];
    }
  }
}

void BatchEngine::polish(sankhya_gb300_batch_item* items, sankhya_gb300_adjoint_info* info) {
  Trace trace("batch polish");
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  ensure_adjoint_buffers();
  AdjointBuffers a = adjoint_buffers();
  SGB_CUDA(cudaMemsetAsync(d_queue_.ptr + 3, 0, sizeof(unsigned int), s));
  const int grid =
      std::max(1, std::min(count_, num_sms_ * adjoint_blocks_per_sm(a.smem_vec)));
  launch_batch_polish(buffers_, a, grid, s);
  SGB_CUDA(cudaGetLastError());
  std::vector<BatchOutcome> out(static_cast<size_t>(count_));
  std::vector<AdjointOutcome> pol(static_cast<size_t>(count_));
  SGB_CUDA(cudaMemcpyAsync(out.data(), outcome_.ptr, out.size() * sizeof(BatchOutcome),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaMemcpyAsync(pol.data(), a_out_.ptr, pol.size() * sizeof(AdjointOutcome),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < count_; ++k) {
    const BatchOutcome& o = out[static_cast<size_t>(k)];
    if (items != nullptr) {
      sankhya_gb300_batch_item& it = items[k];
      it.status = o.status;
      it.objective = o.objective;
      it.dual_bound = o.dual_bound;
      const Residuals& f = o.final_residuals;
      it.final_residuals = sankhya_gb300_residuals{f.primal,          f.dual,           f.gap,
                                                   f.primal_objective, f.dual_objective,
                                                   f.absolute_primal,  f.absolute_dual,
                                                   f.gap_as_verified,  f.complementarity};
    }
    if (info != nullptr) {
      const AdjointOutcome& p = pol[static_cast<size_t>(k)];
      info[k].status = p.status;
      info[k].basic_cols = p.basic_cols;
      info[k].active_rows = p.active_rows;
      info[k].iterations[0] = p.iterations[0];
      info[k].iterations[1] = p.iterations[1];
      info[k].residual[0] = p.residual[0];
      info[k].residual[1] = p.residual[1];
    }
  }
}

}  // namespace sgb

// qp.cu -- host driver of the convex-QP engine.
//
// Follows sankhya::qp::solve_convex_qp (src/qp/qp_condat_vu.cpp:164-362) after its
// convexity gate, with every vector on the device:
//   setup   ||A|| and ||Q|| by the reference's two 20-step power iterations from its
//           std::mt19937 starts (:74-143), on the device; tau and sigma by its formula with
//           the 5% margin (:195-208), on the host; x0 = proj(0), y0 = 0 (:213-225);
//   loop    CUDA graphs of `periods` check periods, each 50 iterations (column pass + row
//           pass) and the check (row pass on A x, column pass on the gradient, decision);
//           the host reads the control block after each graph;
//   report  col_dual = c + Qx + sense A'y, row_dual = -sense y, the objective (:341-361).
// The reference tests the clock before every iteration and the stop controller every 50;
// this engine tests both, and the interrupt flag and poll callback, after every graph.
#include "qp_engine.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

namespace sgb {
namespace {

double qp_now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

std::string qp_format(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return buf;
}

bool valid_lanes(int g) { return g == 1 || g == 2 || g == 4 || g == 8 || g == 16 || g == 32; }

}  // namespace

QpEngine::QpEngine(int device) : device_(device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "no CUDA device " + std::to_string(device)};
  }
  SGB_CUDA(cudaSetDevice(device));
  SGB_CUDA(qp_configure_kernels());
  SGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SGB_CUDA(cudaMallocHost(&ctl_host_, sizeof(QpCtl)));
  SGB_CUDA(cudaMallocHost(&hist_host_, sizeof(QpHist) * kQpMaxPeriods));
  ctl_.allocate(1);
  hist_.allocate(kQpMaxPeriods);
  dot_part_.allocate(kQpDotBlocks);
  dot_out_.allocate(1);
}

QpEngine::~QpEngine() {
  cudaSetDevice(device_);
  destroy_graph();
  if (ctl_host_ != nullptr) cudaFreeHost(ctl_host_);
  if (hist_host_ != nullptr) cudaFreeHost(hist_host_);
  if (stream_ != nullptr) cudaStreamDestroy(stream_);
}

void QpEngine::require_loaded() const {
  if (!loaded_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no QP has been loaded"};
}

void QpEngine::destroy_graph() {
  if (graph_ != nullptr) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
  graph_periods_ = 0;
}

void QpEngine::load(const sankhya_gb300_qp_problem& p) {
  Trace trace("qp load");
  const sankhya_gb300_lp& lp = p.lp;
  validate_lp(lp);
  const int m = lp.rows, n = lp.cols;
  const long long nnz = lp.col_starts[n];
  // The Hessian: well-formed CSC of n x n, finite values, and no diagonal entry that is
  // negative in minimisation sense (the first certificate of src/qp/convexity.cpp:89-100).
  long long hz = 0;
  const double sense = lp.sense < 0.0 ? -1.0 : 1.0;
  if (p.hessian_starts != nullptr) {
    if (p.hessian_starts[0] != 0) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL, "Hessian column starts must begin at 0"};
    }
    for (int j = 0; j < n; ++j) {
      if (p.hessian_starts[j + 1] < p.hessian_starts[j]) {
        throw EngineError{SANKHYA_GB300_ERROR_MODEL, "Hessian column starts are not monotone"};
      }
    }
    hz = p.hessian_starts[n];
    if (hz > 0 && (p.hessian_index == nullptr || p.hessian_values == nullptr)) {
      throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "null Hessian arrays"};
    }
    double largest = 0.0;
    for (int j = 0; j < n; ++j) {
      for (int k = p.hessian_starts[j]; k < p.hessian_starts[j + 1]; ++k) {
        const int i = p.hessian_index[k];
        const double v = p.hessian_values[k];
        if (i < 0 || i >= n) {
          throw EngineError{SANKHYA_GB300_ERROR_MODEL,
                            qp_format("Hessian row index %d out of range", i)};
        }
        if (!std::isfinite(v)) {
          throw EngineError{SANKHYA_GB300_ERROR_MODEL,
                            qp_format("Hessian entry (%d, %d) is not finite", i, j)};
        }
        if (i == j) largest = std::max(largest, std::fabs(sense * v));
      }
    }
    const double slack = 1e-10 * std::max(1.0, largest);
    for (int j = 0; j < n; ++j) {
      for (int k = p.hessian_starts[j]; k < p.hessian_starts[j + 1]; ++k) {
        if (p.hessian_index[k] == j && sense * p.hessian_values[k] < -slack) {
          throw EngineError{
              SANKHYA_GB300_ERROR_MODEL,
              qp_format("the quadratic objective is not convex: the Hessian diagonal for "
                        "column %d is %.6g in minimization sense",
                        j, sense * p.hessian_values[k])};
        }
      }
    }
  }
  if (hz > std::numeric_limits<int>::max() / 2) {
    throw EngineError{SANKHYA_GB300_ERROR_MODEL, "more Hessian nonzeros than int32 indices address"};
  }

  SGB_CUDA(cudaSetDevice(device_));
  destroy_graph();
  loaded_ = solved_ = false;
  col_lanes_ = row_lanes_ = 0;
  m_ = m;
  n_ = n;
  nnz_a_ = nnz;
  nnz_q_stored_ = hz;
  sense_ = sense;
  offset_ = lp.objective_offset;

  // The host layouts (qp_layout.hpp): A by rows, sense Q by rows with both triangles, the
  // items' lengths, the cost and bounds in the kernels' forms.
  QpHostLayout h;
  qp_build_layout(p, &h);
  const long long qz = static_cast<long long>(h.q_cols.size());
  nnz_q_ = qz;
  col_len_ = h.col_len;
  row_len_ = h.row_len;

  cudaStream_t s = stream_;
  const size_t z = static_cast<size_t>(nnz);
  a_cs_.upload(lp.col_starts, static_cast<size_t>(n) + 1, s);
  a_ri_.upload(lp.row_index, z, s);
  a_cv_.upload(lp.values, z, s);
  a_rs_.upload(h.row_starts.data(), h.row_starts.size(), s);
  a_ci_.upload(h.row_cols.data(), z, s);
  a_rv_.upload(h.row_values.data(), z, s);
  q_rs_.upload(h.q_starts.data(), h.q_starts.size(), s);
  q_ci_.upload(h.q_cols.data(), static_cast<size_t>(qz), s);
  q_v_.upload(h.q_values.data(), static_cast<size_t>(qz), s);
  cost_.upload(h.cost.data(), h.cost.size(), s);
  col_lower_.upload(h.col_lower.data(), h.col_lower.size(), s);
  col_upper_.upload(h.col_upper.data(), h.col_upper.size(), s);
  row_lower_.upload(h.row_lower.data(), h.row_lower.size(), s);
  row_upper_.upload(h.row_upper.data(), h.row_upper.size(), s);
  for (auto* a : {&x0_, &x1_, &xbar_, &col_dual_, &vec_n_}) a->allocate(static_cast<size_t>(n));
  for (auto* a : {&y_, &row_dual_, &vec_m_}) a->allocate(static_cast<size_t>(m));
  SGB_CUDA(cudaStreamSynchronize(s));
  loaded_ = true;
}

void QpEngine::layout(int col_lanes, int row_lanes) {
  if (col_lanes == col_lanes_ && row_lanes == row_lanes_) return;
  cudaStream_t s = stream_;
  std::vector<QpChunk> cc, rc;
  qp_build_chunks(col_len_, col_lanes, &cc, &nlong_cols_);
  qp_build_chunks(row_len_, row_lanes, &rc, &nlong_rows_);
  ncol_chunks_ = static_cast<int>(cc.size());
  nrow_chunks_ = static_cast<int>(rc.size());
  col_chunks_.upload(cc.data(), cc.size(), s);
  row_chunks_.upload(rc.data(), rc.size(), s);
  col_part_.allocate(cc.size());
  row_part_.allocate(rc.size());
  col_tickets_.allocate_padded(static_cast<size_t>(nlong_cols_), 1, s);
  row_tickets_.allocate_padded(static_cast<size_t>(nlong_rows_), 1, s);
  long_col_obj_.allocate_padded(static_cast<size_t>(nlong_cols_), 1, s);
  col_short_blocks_ = static_cast<int>((static_cast<long long>(n_) * col_lanes + kQpThreads - 1) /
                                       kQpThreads);
  row_short_blocks_ = static_cast<int>((static_cast<long long>(m_) * row_lanes + kQpThreads - 1) /
                                       kQpThreads);
  obj_part_.allocate_padded(static_cast<size_t>(col_short_blocks_), 1, s);
  SGB_CUDA(cudaStreamSynchronize(s));
  col_lanes_ = col_lanes;
  row_lanes_ = row_lanes;
  destroy_graph();
}

QpDev QpEngine::dev() const {
  QpDev d{};
  d.m = m_;
  d.n = n_;
  d.col_lanes = col_lanes_;
  d.row_lanes = row_lanes_;
  d.stage = stage_;
  d.sense = sense_;
  d.offset = offset_;
  d.a_cs = a_cs_.ptr;
  d.a_ri = a_ri_.ptr;
  d.a_cv = a_cv_.ptr;
  d.a_rs = a_rs_.ptr;
  d.a_ci = a_ci_.ptr;
  d.a_rv = a_rv_.ptr;
  d.q_rs = q_rs_.ptr;
  d.q_ci = q_ci_.ptr;
  d.q_v = q_v_.ptr;
  d.cost = cost_.ptr;
  d.col_lower = col_lower_.ptr;
  d.col_upper = col_upper_.ptr;
  d.row_lower = row_lower_.ptr;
  d.row_upper = row_upper_.ptr;
  d.x0 = x0_.ptr;
  d.x1 = x1_.ptr;
  d.xbar = xbar_.ptr;
  d.y = y_.ptr;
  d.col_dual = col_dual_.ptr;
  d.col_chunks = col_chunks_.ptr;
  d.ncol_chunks = ncol_chunks_;
  d.row_chunks = row_chunks_.ptr;
  d.nrow_chunks = nrow_chunks_;
  d.chunk_part = col_part_.ptr;
  d.row_chunk_part = row_part_.ptr;
  d.col_tickets = col_tickets_.ptr;
  d.row_tickets = row_tickets_.ptr;
  d.long_col_obj = long_col_obj_.ptr;
  d.nlong_cols = nlong_cols_;
  d.obj_part = obj_part_.ptr;
  d.col_short_blocks = col_short_blocks_;
  d.row_short_blocks = row_short_blocks_;
  d.hist = hist_.ptr;
  return d;
}

double QpEngine::dot(const double* a, const double* b, int n) {
  qp_launch_dot(a, b, n, dot_part_.ptr, dot_out_.ptr, stream_);
  double out = 0.0;
  SGB_CUDA(cudaMemcpyAsync(&out, dot_out_.ptr, sizeof(double), cudaMemcpyDeviceToHost, stream_));
  SGB_CUDA(cudaStreamSynchronize(stream_));
  return out;
}

// ||A||: src/qp/qp_condat_vu.cpp:74-103 (std::mt19937(26119 + seed), uniform on [-1, 1],
// twenty steps of v <- A'A v / |v|, estimate |A'A v|^(1/2)).
double QpEngine::spectral_norm(unsigned seed) {
  if (m_ == 0 || n_ == 0 || nnz_a_ == 0) return 0.0;
  std::mt19937 rng(26119u + seed);
  std::uniform_real_distribution<double> unit(-1.0, 1.0);
  std::vector<double> v(static_cast<size_t>(n_));
  for (double& value : v) value = unit(rng);
  SGB_CUDA(cudaMemcpyAsync(vec_n_.ptr, v.data(), v.size() * sizeof(double),
                           cudaMemcpyHostToDevice, stream_));
  double estimate = 0.0;
  for (int iteration = 0; iteration < 20; ++iteration) {
    const double norm2 = dot(vec_n_.ptr, vec_n_.ptr, n_);
    if (std::sqrt(norm2) <= 0.0) return 0.0;
    qp_launch_scale(vec_n_.ptr, n_, dot_out_.ptr, stream_);
    qp_launch_spmv(m_, a_rs_.ptr, a_ci_.ptr, a_rv_.ptr, vec_n_.ptr, vec_m_.ptr,
                   qp_auto_lanes(double(nnz_a_) / m_), stream_);
    qp_launch_spmv(n_, a_cs_.ptr, a_ri_.ptr, a_cv_.ptr, vec_m_.ptr, vec_n_.ptr,
                   qp_auto_lanes(double(nnz_a_) / n_), stream_);
    estimate = std::sqrt(std::sqrt(dot(vec_n_.ptr, vec_n_.ptr, n_)));
  }
  return estimate;
}

// ||Q||: src/qp/qp_condat_vu.cpp:105-143 (std::mt19937(20260826 + seed), twenty steps of
// v <- Q v / |v|, estimate |v' Q v| for the normalised v).
double QpEngine::hessian_norm(unsigned seed) {
  if (nnz_q_stored_ == 0 || n_ == 0) return 0.0;
  std::mt19937 rng(20260826u + seed);
  std::uniform_real_distribution<double> unit(-1.0, 1.0);
  std::vector<double> v(static_cast<size_t>(n_));
  for (double& value : v) value = unit(rng);
  SGB_CUDA(cudaMemcpyAsync(vec_n_.ptr, v.data(), v.size() * sizeof(double),
                           cudaMemcpyHostToDevice, stream_));
  double* a = vec_n_.ptr;
  double* b = col_dual_.ptr;  // scratch until the report
  double estimate = 0.0;
  for (int iteration = 0; iteration < 20; ++iteration) {
    const double norm2 = dot(a, a, n_);
    if (std::sqrt(norm2) <= 0.0) return 0.0;
    qp_launch_scale(a, n_, dot_out_.ptr, stream_);
    qp_launch_spmv(n_, q_rs_.ptr, q_ci_.ptr, q_v_.ptr, a, b, qp_auto_lanes(double(nnz_q_) / n_),
                   stream_);
    estimate = std::fabs(dot(b, a, n_));
    std::swap(a, b);
  }
  return estimate;
}

void QpEngine::build_graph(int periods) {
  if (graph_ != nullptr && graph_periods_ == periods && graph_col_lanes_ == col_lanes_ &&
      graph_row_lanes_ == row_lanes_ && graph_stage_ == stage_) {
    return;
  }
  destroy_graph();
  const QpDev d = dev();
  QpCtl* ctl = ctl_.ptr;
  const long long before = qp_kernel_launch_count();
  cudaGraph_t graph = nullptr;
  SGB_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
  for (int p = 0; p < periods; ++p) {
    for (int it = 0; it < kQpCheckEvery; ++it) {
      const int k = p * kQpCheckEvery + it;
      qp_launch_column_pass(d, ctl, kQpStep, k, k & 1, stream_);
      if (m_ > 0) qp_launch_row_pass(d, ctl, kQpStep, k, 0, stream_);
    }
    // After an even number of iterations x is back in buffer 0.
    const int last = p * kQpCheckEvery + kQpCheckEvery - 1;
    if (m_ > 0) qp_launch_row_pass(d, ctl, kQpCheck, last, 0, stream_);
    qp_launch_column_pass(d, ctl, kQpCheck, last, 0, stream_);
    qp_launch_decide(d, ctl, last, p, stream_);
  }
  qp_launch_advance(ctl, periods * kQpCheckEvery, stream_);
  const cudaError_t end = cudaStreamEndCapture(stream_, &graph);
  SGB_CUDA(end);
  const cudaError_t inst = cudaGraphInstantiate(&graph_, graph, 0);
  cudaGraphDestroy(graph);
  SGB_CUDA(inst);
  graph_nodes_ = qp_kernel_launch_count() - before;
  graph_periods_ = periods;
  graph_col_lanes_ = col_lanes_;
  graph_row_lanes_ = row_lanes_;
  graph_stage_ = stage_;
}

void QpEngine::solve(const sankhya_gb300_qp_params& p, sankhya_gb300_qp_result* r) {
  Trace trace("qp solve");
  const double t0 = qp_now();
  require_loaded();
  std::memset(r, 0, sizeof(*r));
  if (!(p.tolerance > 0.0) || std::isnan(p.time_limit)) {
    throw EngineError{SANKHYA_GB300_ERROR_OPTION, "qp_tolerance must be positive"};
  }
  const int col_lanes = p.column_lanes > 0 ? p.column_lanes
                                           : qp_auto_lanes(n_ > 0 ? double(nnz_a_ + nnz_q_) / n_ : 1.0);
  const int row_lanes = p.row_lanes > 0 ? p.row_lanes
                                        : qp_auto_lanes(m_ > 0 ? double(nnz_a_) / m_ : 1.0);
  if (!valid_lanes(col_lanes) || !valid_lanes(row_lanes)) {
    throw EngineError{SANKHYA_GB300_ERROR_OPTION, "lanes must be 1, 2, 4, 8, 16 or 32"};
  }
  SGB_CUDA(cudaSetDevice(device_));
  solved_ = false;
  layout(col_lanes, row_lanes);
  stage_ = p.staging ? 1 : 0;
  // Check periods per graph: about 2 ms of work by the bytes an iteration moves, at most 20.
  int periods = p.periods_per_poll;
  if (periods <= 0) {
    const double bytes = 12.0 * (2.0 * double(nnz_a_) + double(nnz_q_)) + 8.0 * (8.0 * n_ + 6.0 * m_);
    const double per_iteration = bytes / 4e12 + 6e-6;
    periods = static_cast<int>(std::ceil(2e-3 / (kQpCheckEvery * per_iteration)));
    periods = std::max(1, std::min(periods, 20));
  }
  periods = std::min(periods, kQpMaxPeriods);
  const long long launches_before = qp_kernel_launch_count();

  cudaEvent_t ev[4];
  for (auto& e : ev) SGB_CUDA(cudaEventCreate(&e));
  struct EventGuard {
    cudaEvent_t* e;
    ~EventGuard() {
      for (int k = 0; k < 4; ++k) cudaEventDestroy(e[k]);
    }
  } guard{ev};
  SGB_CUDA(cudaEventRecord(ev[0], stream_));

  // Step sizes (src/qp/qp_condat_vu.cpp:195-208).
  const auto seed = static_cast<unsigned>(p.random_seed);
  const double norm_a = spectral_norm(seed);
  const double norm_q = hessian_norm(seed);
  const double margin = 1.05;
  const double l = margin * norm_q;
  const double a2 = margin * margin * std::max(norm_a * norm_a, 1e-12);
  const double tau = 1.0 / (l / 2.0 + std::sqrt(a2) + 1e-12);
  const double sigma = (m_ > 0) ? (1.0 / tau - l / 2.0) / (2.0 * a2) : 0.0;
  r->norm_a = norm_a;
  r->norm_q = norm_q;
  r->tau = tau;
  r->sigma = sigma;
  r->column_lanes = col_lanes;
  r->row_lanes = row_lanes;

  const QpDev d = dev();
  qp_launch_init(d, stream_);
  SGB_CUDA(cudaMemsetAsync(hist_.ptr, 0, sizeof(QpHist) * kQpMaxPeriods, stream_));
  const bool ceiling = p.iteration_limit < 0;
  QpCtl c{};
  c.tau = tau;
  c.sigma = sigma;
  c.inv_sigma = sigma > 0.0 ? 1.0 / sigma : 0.0;
  c.tolerance = p.tolerance;
  c.limit = ceiling ? 1000000 : p.iteration_limit;
  SGB_CUDA(cudaMemcpyAsync(ctl_.ptr, &c, sizeof(QpCtl), cudaMemcpyHostToDevice, stream_));
  SGB_CUDA(cudaEventRecord(ev[1], stream_));
  const long long launches_setup = qp_kernel_launch_count() - launches_before;
  build_graph(periods);

  int status = SANKHYA_GB300_ITERATION_LIMIT;
  long long base = 0, graphs = 0;
  const double time_limit = p.time_limit;
  *ctl_host_ = c;
  for (;;) {
    const double elapsed = qp_now() - t0;
    if (time_limit < 1e300 && (time_limit <= 0.0 || elapsed > time_limit)) {
      status = SANKHYA_GB300_TIME_LIMIT;
      break;
    }
    if (base >= c.limit) {
      status = SANKHYA_GB300_ITERATION_LIMIT;
      r->ceiling = ceiling ? 1 : 0;
      break;
    }
    SGB_CUDA(cudaGraphLaunch(graph_, stream_));
    ++graphs;
    SGB_CUDA(cudaMemcpyAsync(ctl_host_, ctl_.ptr, sizeof(QpCtl), cudaMemcpyDeviceToHost,
                             stream_));
    SGB_CUDA(cudaMemcpyAsync(hist_host_, hist_.ptr, sizeof(QpHist) * periods,
                             cudaMemcpyDeviceToHost, stream_));
    SGB_CUDA(cudaStreamSynchronize(stream_));
    const QpCtl now = *ctl_host_;
    // The reference logs every 5,000 iterations at a check that did not stop the loop
    // (src/qp/qp_condat_vu.cpp:327-330).
    if (p.log != nullptr) {
      for (int q = 0; q < periods; ++q) {
        const QpHist h = hist_host_[q];
        if (h.iteration <= base || h.iteration % 5000 != 0) continue;
        if (now.done && h.iteration == now.iterations) continue;
        p.log(p.log_user, h.iteration, h.objective, h.primal, h.dual, qp_now() - t0);
      }
    }
    base = now.base;
    if (now.done) {
      status = SANKHYA_GB300_OPTIMAL;
      base = now.iterations;
      break;
    }
    if ((p.interrupt != nullptr && *p.interrupt != 0) ||
        (p.poll != nullptr && p.poll(p.poll_user, base, now.objective) != 0)) {
      status = SANKHYA_GB300_INTERRUPTED;
      break;
    }
  }
  SGB_CUDA(cudaEventRecord(ev[2], stream_));
  final_iterations_ = base;

  // Report: col_dual and the objective at the reported x, row_dual.
  const long long launches_report = qp_kernel_launch_count();
  qp_launch_column_pass(d, ctl_.ptr, kQpReport, 0, static_cast<int>(base & 1), stream_);
  qp_launch_row_dual(d, row_dual_.ptr, stream_);
  SGB_CUDA(cudaMemcpyAsync(ctl_host_, ctl_.ptr, sizeof(QpCtl), cudaMemcpyDeviceToHost, stream_));
  SGB_CUDA(cudaEventRecord(ev[3], stream_));
  SGB_CUDA(cudaStreamSynchronize(stream_));
  const QpCtl fin = *ctl_host_;
  float ms_setup = 0.f, ms_loop = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_setup, ev[0], ev[1]);
  cudaEventElapsedTime(&ms_loop, ev[1], ev[2]);
  cudaEventElapsedTime(&ms_all, ev[0], ev[3]);

  r->status = status;
  r->iterations = base;
  r->primal_residual = fin.checked > 0 ? fin.primal : -1.0;
  r->dual_residual = fin.checked > 0 ? fin.dual : -1.0;
  r->objective = fin.objective;
  r->setup_seconds = 1e-3 * ms_setup;
  r->loop_seconds = 1e-3 * ms_loop;
  r->device_seconds = 1e-3 * ms_all;
  r->kernel_launches = launches_setup + graphs * graph_nodes_ +
                       (qp_kernel_launch_count() - launches_report);
  const char* what = status == SANKHYA_GB300_OPTIMAL      ? "optimal"
                     : status == SANKHYA_GB300_TIME_LIMIT ? "time limit"
                     : status == SANKHYA_GB300_INTERRUPTED ? "interrupted"
                                                           : "iteration limit";
  std::snprintf(r->message, sizeof(r->message),
                "%s after %lld iterations: primal residual %.3e, dual residual %.3e "
                "(tolerance %.1e)%s",
                what, base, r->primal_residual, r->dual_residual, p.tolerance,
                r->ceiling ? "; the engine's own ceiling of 1000000 iterations" : "");
  solved_ = true;
  r->solve_seconds = qp_now() - t0;
}

void QpEngine::solution(double* col_value, double* col_dual, double* row_dual) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no QP solve has run"};
  SGB_CUDA(cudaSetDevice(device_));
  const double* x = (final_iterations_ & 1) ? x1_.ptr : x0_.ptr;
  const size_t n = static_cast<size_t>(n_), m = static_cast<size_t>(m_);
  if (col_value != nullptr && n > 0) {
    SGB_CUDA(cudaMemcpyAsync(col_value, x, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  }
  if (col_dual != nullptr && n > 0) {
    SGB_CUDA(cudaMemcpyAsync(col_dual, col_dual_.ptr, n * sizeof(double),
                             cudaMemcpyDeviceToHost, stream_));
  }
  if (row_dual != nullptr && m > 0) {
    SGB_CUDA(cudaMemcpyAsync(row_dual, row_dual_.ptr, m * sizeof(double),
                             cudaMemcpyDeviceToHost, stream_));
  }
  SGB_CUDA(cudaStreamSynchronize(stream_));
}

void QpEngine::time_kernels(int reps, double* ms) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no QP solve has run"};
  if (reps <= 0) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "reps must be positive"};
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  const size_t n = static_cast<size_t>(n_), m = static_cast<size_t>(m_);
  // Keep the solve's state: both x buffers, xbar, y and the control block.
  DeviceArray<double> keep;
  keep.allocate(3 * n + m + 1);
  SGB_CUDA(cudaMemcpyAsync(keep.ptr, x0_.ptr, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(keep.ptr + n, x1_.ptr, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(keep.ptr + 2 * n, xbar_.ptr, n * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(keep.ptr + 3 * n, y_.ptr, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  QpCtl saved{};
  SGB_CUDA(cudaMemcpyAsync(&saved, ctl_.ptr, sizeof(QpCtl), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  QpCtl run = saved;
  run.done = 0;
  run.base = 0;
  run.limit = std::numeric_limits<long long>::max() / 2;
  SGB_CUDA(cudaMemcpyAsync(ctl_.ptr, &run, sizeof(QpCtl), cudaMemcpyHostToDevice, s));
  const QpDev d = dev();
  std::vector<cudaEvent_t> ev(3 * static_cast<size_t>(reps));
  for (auto& e : ev) SGB_CUDA(cudaEventCreate(&e));
  int src = static_cast<int>(final_iterations_ & 1);
  for (int q = 0; q < reps; ++q) {
    SGB_CUDA(cudaEventRecord(ev[3 * q], s));
    qp_launch_column_pass(d, ctl_.ptr, kQpStep, 0, src, s);
    SGB_CUDA(cudaEventRecord(ev[3 * q + 1], s));
    if (m_ > 0) qp_launch_row_pass(d, ctl_.ptr, kQpStep, 0, 0, s);
    SGB_CUDA(cudaEventRecord(ev[3 * q + 2], s));
    src ^= 1;
  }
  SGB_CUDA(cudaStreamSynchronize(s));
  double col = 0.0, row = 0.0;
  for (int q = 0; q < reps; ++q) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, ev[3 * q], ev[3 * q + 1]);
    cudaEventElapsedTime(&b, ev[3 * q + 1], ev[3 * q + 2]);
    col += a;
    row += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  ms[0] = col / reps;
  ms[1] = row / reps;
  SGB_CUDA(cudaMemcpyAsync(x0_.ptr, keep.ptr, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(x1_.ptr, keep.ptr + n, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(xbar_.ptr, keep.ptr + 2 * n, n * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(y_.ptr, keep.ptr + 3 * n, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SGB_CUDA(cudaMemcpyAsync(ctl_.ptr, &saved, sizeof(QpCtl), cudaMemcpyHostToDevice, s));
  SGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sgb

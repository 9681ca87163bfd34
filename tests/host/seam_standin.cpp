// seam_standin.cpp -- a CPU stand-in for the engine's C ABI, for the seam's behaviour test.
//
// Implements the five calls seam/pdhg_gpu.cpp makes (create, load, solve, solution,
// last_error) by handing the LP to the REFERENCE's own CPU PDHG (sankhya::pdhg::solve_pdhg,
// compiled from the reference's sources) with the options rebuilt from the params struct the
// seam filled in. The seam is then checked against a direct call of the same reference
// function: every option row it forwards, every field it fills and every status it maps must
// come out the same. It also drives the seam's hooks: one iteration-table row through
// params.log, the interrupt through params.poll, and a failing create on request
// (standin_fail_create).
//
// For the front-end test it also answers the device probes and the memory estimate that
// seam/device.cpp and seam/gpu_memory.cpp forward to the C ABI, with a device the test sets
// (standin_set_device), and counts the solves it ran (standin_solve_count), so a test can
// tell whether SANKHYA's solve() reached the seam or took its own CPU path. Test
// infrastructure only; nothing here is part of the engine.
//
// The QP calls seam/qp_gpu.cpp makes (qp create, load, solve, solution) hand the QP to the
// reference's own CPU engine, sankhya::qp::solve_convex_qp, with the options rebuilt from the
// params struct.
//
// The batched calls seam/node_batch.cpp makes (batch create, load, solve, solution, ray) are
// answered the same way, one reference solve per LP. The reference's PDHG detects no
// infeasibility, so a test marks an LP infeasible itself, with the direction the stand-in
// returns as its certificate (standin_batch_mark_infeasible).
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/pdhg.hpp"
#include "sankhya/qp.hpp"
#include "sankhya_gb300.h"

struct sankhya_gb300_pdhg {
  sankhya::Model model;
  sankhya::Solution solution;
  bool solved = false;
};

struct sankhya_gb300_batch {
  std::vector<sankhya::Model> models;
  std::vector<sankhya::Solution> solutions;
  bool solved = false;
};

struct sankhya_gb300_qp {
  sankhya::Model model;
  sankhya::Solution solution;
  bool solved = false;
};

namespace {

thread_local std::string g_error;
std::map<int, std::vector<double>> g_infeasible;  // LP index -> its certificate
int g_fail_create = 0;
std::atomic<long long> g_solves{0};

// The device the probes describe: a GB300 with 280 GiB free, unless a test says otherwise.
struct Device {
  int available = 1;
  int major = 10;
  int minor = 3;
  unsigned long long free_bytes = 280ULL << 30;
  unsigned long long total_bytes = 284ULL << 30;
  unsigned long long estimate = 64ULL << 20;
};
Device g_device;

int32_t to_code(sankhya::SolveStatus s) {
  using S = sankhya::SolveStatus;
  switch (s) {
    case S::kOptimal: return SANKHYA_GB300_OPTIMAL;
    case S::kFeasible: return SANKHYA_GB300_FEASIBLE;
    case S::kInfeasible: return SANKHYA_GB300_INFEASIBLE;
    case S::kIterationLimit: return SANKHYA_GB300_ITERATION_LIMIT;
    case S::kTimeLimit: return SANKHYA_GB300_TIME_LIMIT;
    case S::kInterrupted: return SANKHYA_GB300_INTERRUPTED;
    case S::kModelError: return SANKHYA_GB300_MODEL_ERROR;
    default: return SANKHYA_GB300_NUMERICAL_ERROR;
  }
}

sankhya::Options options_of(const sankhya_gb300_params* p) {
  sankhya::Options o;
  o.set_double("pdhg_tolerance", p->tolerance);
  o.set_int("iteration_limit", p->iteration_limit);
  o.set_double("time_limit", p->time_limit);
  o.set_bool("pdhg_restart", p->restart != 0);
  o.set_bool("pdhg_stop_at_request", p->stop_at_request != 0);
  o.set_int("random_seed", p->random_seed);
  return o;
}

void to_model(const sankhya_gb300_lp* lp, sankhya::Model& m) {
  m = sankhya::Model();
  const auto n = static_cast<std::size_t>(lp->cols);
  const auto rows = static_cast<std::size_t>(lp->rows);
  m.sense = lp->sense < 0.0 ? sankhya::ObjSense::kMaximize : sankhya::ObjSense::kMinimize;
  m.objective_offset = lp->objective_offset;
  m.col_cost.assign(lp->col_cost, lp->col_cost + n);
  m.col_lower.assign(lp->col_lower, lp->col_lower + n);
  m.col_upper.assign(lp->col_upper, lp->col_upper + n);
  m.col_type.assign(n, sankhya::VarType::kContinuous);
  m.row_lower.assign(lp->row_lower, lp->row_lower + rows);
  m.row_upper.assign(lp->row_upper, lp->row_upper + rows);
  m.matrix.reset(lp->rows, lp->cols);
  for (int32_t j = 0; j < lp->cols; ++j) {
    for (int32_t k = lp->col_starts[j]; k < lp->col_starts[j + 1]; ++k) {
      m.matrix.add_entry(lp->row_index[k], j, lp->values[k]);
    }
  }
  m.matrix.finalize(0.0);
}

}  // namespace

extern "C" {

void standin_fail_create(int fail) { g_fail_create = fail; }

void standin_set_device(int available, int major, int minor, unsigned long long free_bytes,
                        unsigned long long total_bytes, unsigned long long estimate) {
  g_device = Device{available, major, minor, free_bytes, total_bytes, estimate};
}

long long standin_solve_count(void) { return g_solves.load(); }

int sankhya_gb300_device_available(char* description, int32_t capacity) {
  if (description != nullptr && capacity > 0) {
    std::snprintf(description, static_cast<std::size_t>(capacity), "%s",
                  g_device.available ? "NVIDIA GB300 (stand-in)" : "no device (stand-in)");
  }
  return g_device.available ? SANKHYA_GB300_OK : SANKHYA_GB300_ERROR_DEVICE;
}

int sankhya_gb300_device_free_memory(size_t* free_bytes, size_t* total_bytes) {
  if (!g_device.available) return SANKHYA_GB300_ERROR_DEVICE;
  if (free_bytes != nullptr) *free_bytes = static_cast<size_t>(g_device.free_bytes);
  if (total_bytes != nullptr) *total_bytes = static_cast<size_t>(g_device.total_bytes);
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_device_compute_capability(int32_t* major, int32_t* minor) {
  if (!g_device.available) return SANKHYA_GB300_ERROR_DEVICE;
  if (major != nullptr) *major = g_device.major;
  if (minor != nullptr) *minor = g_device.minor;
  return SANKHYA_GB300_OK;
}

size_t sankhya_gb300_estimate_memory(int32_t rows, int32_t cols, int64_t nonzeros,
                                     int32_t precision) {
  (void)rows;
  (void)cols;
  (void)nonzeros;
  (void)precision;
  return static_cast<size_t>(g_device.estimate);
}

const char* sankhya_gb300_last_error(void) { return g_error.c_str(); }

int sankhya_gb300_pdhg_create(int32_t device, sankhya_gb300_pdhg** out) {
  (void)device;
  if (g_fail_create) {
    g_error = "no usable CUDA device (stand-in)";
    return SANKHYA_GB300_ERROR_DEVICE;
  }
  *out = new sankhya_gb300_pdhg();
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_pdhg_load(sankhya_gb300_pdhg* e, const sankhya_gb300_lp* lp) {
  to_model(lp, e->model);
  e->solved = false;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_pdhg_solve(sankhya_gb300_pdhg* e, const sankhya_gb300_params* p,
                             sankhya_gb300_result* r) {
  std::memset(r, 0, sizeof(*r));
  if (p->poll != nullptr && p->poll(p->poll_user, 0, 0.0) != 0) {
    e->solution = sankhya::Solution();
    e->solution.allocate_for(e->model);
    e->solved = true;
    r->status = SANKHYA_GB300_INTERRUPTED;
    std::strncpy(r->message, "interrupted (stand-in)", sizeof(r->message) - 1);
    return SANKHYA_GB300_OK;
  }
  if (p->precision != SANKHYA_GB300_FP64 || p->stop_rule != SANKHYA_GB300_STOP_STANDARD) {
    g_error = "the stand-in runs the reference method only";
    return SANKHYA_GB300_ERROR_OPTION;
  }
  const sankhya::Options o = options_of(p);
  sankhya::Logger quiet(nullptr);
  e->solution = sankhya::pdhg::solve_pdhg(e->model, o, quiet, nullptr);
  e->solved = true;
  ++g_solves;
  if (p->log != nullptr) p->log(p->log_user, 40, e->solution.objective, 1e-3, 2e-3, 0.25);
  r->status = to_code(e->solution.status);
  r->iterations = e->solution.iterations;
  // The restart count is not a Solution field; the engine's message carries it
  // ("... after N iterations and R restarts ...", src/pdhg/pdhg.cpp:519-548). Every step of
  // the CPU engine counts as one attempt here, and its time as the loop's.
  const std::size_t at = e->solution.message.find(" iterations and ");
  r->restarts = at == std::string::npos
                    ? 0
                    : std::atoll(e->solution.message.c_str() + at + std::strlen(" iterations and "));
  r->attempts = e->solution.iterations;
  r->loop_seconds = e->solution.solve_seconds;
  r->objective = e->solution.objective;
  r->dual_bound = e->solution.dual_bound;
  r->solve_seconds = e->solution.solve_seconds;
  std::strncpy(r->message, e->solution.message.c_str(), sizeof(r->message) - 1);
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_pdhg_solution(sankhya_gb300_pdhg* e, double* col_value, double* col_dual,
                                double* row_dual) {
  if (!e->solved) {
    g_error = "no solve has run";
    return SANKHYA_GB300_ERROR_ARGUMENT;
  }
  const auto& s = e->solution;
  for (std::size_t j = 0; j < s.col_value.size(); ++j) {
    if (col_value) col_value[j] = s.col_value[j];
    if (col_dual) col_dual[j] = s.col_dual[j];
  }
  for (std::size_t i = 0; i < s.row_dual.size(); ++i) {
    if (row_dual) row_dual[i] = s.row_dual[i];
  }
  return SANKHYA_GB300_OK;
}

void standin_batch_mark_infeasible(int index, const double* ray, int rows) {
  g_infeasible[index] = std::vector<double>(ray, ray + rows);
}

void standin_batch_clear_marks(void) { g_infeasible.clear(); }

int sankhya_gb300_batch_create(int32_t device, sankhya_gb300_batch** out) {
  (void)device;
  if (g_fail_create) {
    g_error = "no usable CUDA device (stand-in)";
    return SANKHYA_GB300_ERROR_DEVICE;
  }
  *out = new sankhya_gb300_batch();
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_batch_destroy(sankhya_gb300_batch* b) {
  delete b;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_batch_load(sankhya_gb300_batch* b, int32_t count, const sankhya_gb300_lp* lps) {
  b->models.assign(static_cast<std::size_t>(count), sankhya::Model());
  for (int32_t k = 0; k < count; ++k) to_model(&lps[k], b->models[static_cast<std::size_t>(k)]);
  b->solved = false;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_batch_solve(sankhya_gb300_batch* b, const sankhya_gb300_params* p,
                              sankhya_gb300_batch_item* items, double* device_seconds) {
  if (p->precision != SANKHYA_GB300_FP64 || p->stop_rule != SANKHYA_GB300_STOP_STANDARD) {
    g_error = "the stand-in runs the reference method only";
    return SANKHYA_GB300_ERROR_OPTION;
  }
  const sankhya::Options o = options_of(p);
  sankhya::Logger quiet(nullptr);
  b->solutions.clear();
  for (std::size_t k = 0; k < b->models.size(); ++k) {
    b->solutions.push_back(sankhya::pdhg::solve_pdhg(b->models[k], o, quiet, nullptr));
    ++g_solves;
    const sankhya::Solution& s = b->solutions.back();
    sankhya_gb300_batch_item& it = items[k];
    std::memset(&it, 0, sizeof(it));
    it.status = g_infeasible.count(static_cast<int>(k)) ? SANKHYA_GB300_INFEASIBLE
                                                        : to_code(s.status);
    it.converged = s.status == sankhya::SolveStatus::kOptimal ||
                   s.status == sankhya::SolveStatus::kFeasible;
    it.iterations = s.iterations;
    it.attempts = s.iterations;
    it.objective = s.objective;
    it.dual_bound = s.dual_bound;
  }
  if (device_seconds != nullptr) *device_seconds = 0.0;
  b->solved = true;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_batch_solution(sankhya_gb300_batch* b, int32_t index, double* col_value,
                                 double* col_dual, double* row_dual) {
  if (!b->solved || index < 0 || static_cast<std::size_t>(index) >= b->solutions.size()) {
    g_error = "no such solved LP";
    return SANKHYA_GB300_ERROR_ARGUMENT;
  }
  const auto& s = b->solutions[static_cast<std::size_t>(index)];
  for (std::size_t j = 0; j < s.col_value.size(); ++j) {
    if (col_value) col_value[j] = s.col_value[j];
    if (col_dual) col_dual[j] = s.col_dual[j];
  }
  for (std::size_t i = 0; i < s.row_dual.size(); ++i) {
    if (row_dual) row_dual[i] = s.row_dual[i];
  }
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_batch_ray(sankhya_gb300_batch* b, int32_t index, double* ray) {
  if (!b->solved || index < 0 || static_cast<std::size_t>(index) >= b->models.size()) {
    g_error = "no such solved LP";
    return SANKHYA_GB300_ERROR_ARGUMENT;
  }
  const std::size_t m = static_cast<std::size_t>(b->models[static_cast<std::size_t>(index)].num_rows());
  const auto found = g_infeasible.find(index);
  for (std::size_t i = 0; i < m; ++i) ray[i] = found != g_infeasible.end() ? found->second[i] : 0.0;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_qp_create(int32_t device, sankhya_gb300_qp** out) {
  (void)device;
  if (g_fail_create) {
    g_error = "no usable CUDA device (stand-in)";
    return SANKHYA_GB300_ERROR_DEVICE;
  }
  *out = new sankhya_gb300_qp();
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_qp_destroy(sankhya_gb300_qp* e) {
  delete e;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_qp_load(sankhya_gb300_qp* e, const sankhya_gb300_qp_problem* p) {
  to_model(&p->lp, e->model);
  e->model.hessian.reset(p->lp.cols, p->lp.cols);
  if (p->hessian_starts != nullptr) {
    for (int32_t j = 0; j < p->lp.cols; ++j) {
      for (int32_t k = p->hessian_starts[j]; k < p->hessian_starts[j + 1]; ++k) {
        e->model.hessian.add_entry(p->hessian_index[k], j, p->hessian_values[k]);
      }
    }
  }
  e->model.hessian.finalize(0.0);
  e->solved = false;
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_qp_solve(sankhya_gb300_qp* e, const sankhya_gb300_qp_params* p,
                           sankhya_gb300_qp_result* r) {
  std::memset(r, 0, sizeof(*r));
  e->solution = sankhya::Solution();
  e->solution.allocate_for(e->model);
  e->solved = true;
  if (p->poll != nullptr && p->poll(p->poll_user, 0, 0.0) != 0) {
    r->status = SANKHYA_GB300_INTERRUPTED;
    return SANKHYA_GB300_OK;
  }
  sankhya::Options o;
  o.set_double("qp_tolerance", p->tolerance);
  o.set_int("iteration_limit", p->iteration_limit);
  o.set_double("time_limit", p->time_limit);
  o.set_int("random_seed", p->random_seed);
  sankhya::Logger quiet(nullptr);
  e->solution = sankhya::qp::solve_convex_qp(e->model, o, quiet, nullptr);
  ++g_solves;
  if (p->log != nullptr) p->log(p->log_user, 5000, e->solution.objective, 1e-3, 2e-3, 0.25);
  r->status = to_code(e->solution.status);
  r->iterations = e->solution.iterations;
  r->objective = e->solution.objective;
  r->solve_seconds = e->solution.solve_seconds;
  std::strncpy(r->message, e->solution.message.c_str(), sizeof(r->message) - 1);
  return SANKHYA_GB300_OK;
}

int sankhya_gb300_qp_solution(sankhya_gb300_qp* e, double* col_value, double* col_dual,
                              double* row_dual) {
  if (!e->solved) {
    g_error = "no solve has run";
    return SANKHYA_GB300_ERROR_ARGUMENT;
  }
  const auto& s = e->solution;
  for (std::size_t j = 0; j < s.col_value.size(); ++j) {
    if (col_value) col_value[j] = s.col_value[j];
    if (col_dual) col_dual[j] = s.col_dual[j];
  }
  for (std::size_t i = 0; i < s.row_dual.size(); ++i) {
    if (row_dual) row_dual[i] = s.row_dual[i];
  }
  return SANKHYA_GB300_OK;
}

}  // extern "C"

// seam_check.cpp -- behaviour of the drop-in seam sankhya::gpu::solve_pdhg_gpu, on the CPU.
//
// Linked with seam/pdhg_gpu.cpp, the C-ABI stand-in (seam_standin.cpp: the reference's CPU
// PDHG behind the engine's calls) and the reference's own compiled sources. For a minimising
// and a maximising LP, with every PDHG option row set away from its default, the seam's
// Solution must equal the reference's solve_pdhg on the same Model and Options: status,
// iterations, message, the three vectors bit for bit, objective, dual bound and the quality
// fields recompute_quality() fills, with algorithm "pdhg-gpu". Then the seam's other paths:
// a Model that fails validation (kModelError before any engine call), an engine that cannot
// be created (kNumericalError with the engine's message, no fallback), an interrupt through
// SolveControl (kInterrupted), and the iteration table written through the Logger. Last,
// four threads solve different Models through the seam at the same time, as callers of
// SANKHYA's solve() may: each must get its own Model's answer, bit for bit. And with a
// profiler on the Logger, the seam reports the same "pdhg restarts" count as the CPU engine
// and its two timed phases.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "gpu/pdhg_gpu.hpp"
#include "sankhya/logging.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/pdhg.hpp"
#include "sankhya/solve_control.hpp"
#include "util/profiler.hpp"

extern "C" void standin_fail_create(int fail);

namespace {

int g_failures = 0;

void check(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what);
    ++g_failures;
  }
}

bool same(const std::vector<double>& a, const std::vector<double>& b) {
  if (a.size() != b.size()) return false;
  for (std::size_t k = 0; k < a.size(); ++k) {
    if (std::memcmp(&a[k], &b[k], sizeof(double)) != 0) return false;
  }
  return true;
}

bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }

// A planted LP: 5 entries per column at distinct random rows, equality rows b = A x0, with a
// few inequality rows and a free column so every bound kind passes through the seam.
sankhya::Model make_model(unsigned seed, bool maximise) {
  std::mt19937 rng(seed);
  std::normal_distribution<double> normal;
  std::uniform_real_distribution<double> unit(0.0, 1.0);
  const int m = 40, n = 90;
  sankhya::Model model;
  model.sense = maximise ? sankhya::ObjSense::kMaximize : sankhya::ObjSense::kMinimize;
  model.objective_offset = 1.25;
  model.matrix.reset(m, n);
  std::vector<double> x0(n), y0(m), ax(m, 0.0), aty(n, 0.0);
  for (int i = 0; i < m; ++i) y0[i] = normal(rng);
  for (int j = 0; j < n; ++j) {
    const double u = unit(rng);
    x0[j] = u < 0.3 ? 0.0 : (u < 0.4 ? 10.0 : 0.1 + 9.8 * unit(rng));
    std::vector<int> rows;
    while (rows.size() < 5) {
      const int r = static_cast<int>(rng() % m);
      bool seen = false;
      for (int q : rows) seen = seen || q == r;
      if (!seen) rows.push_back(r);
    }
    for (int r : rows) {
      const double v = normal(rng);
      model.matrix.add_entry(r, j, v);
      ax[r] += v * x0[j];
      aty[j] += v * y0[r];
    }
  }
  model.matrix.finalize(0.0);
  for (int j = 0; j < n; ++j) {
    const double z = x0[j] == 0.0 ? 0.1 + 0.9 * unit(rng) : (x0[j] == 10.0 ? -0.1 - 0.9 * unit(rng) : 0.0);
    const double c = aty[j] + z;
    model.col_cost.push_back(maximise ? -c : c);
    model.col_lower.push_back(0.0);
    model.col_upper.push_back(10.0);
    model.col_type.push_back(sankhya::VarType::kContinuous);
  }
  for (int i = 0; i < m; ++i) {
    model.row_lower.push_back(ax[i]);
    model.row_upper.push_back(ax[i]);
  }
  return model;
}

sankhya::Options make_options() {
  sankhya::Options o;
  o.set_double("pdhg_tolerance", 1e-6);
  o.set_int("iteration_limit", 20000);
  o.set_double("time_limit", 300.0);
  o.set_bool("pdhg_restart", true);
  o.set_bool("pdhg_stop_at_request", true);
  o.set_int("random_seed", 7);
  return o;
}

void compare(const sankhya::Model& model, const char* label) {
  const sankhya::Options options = make_options();
  sankhya::Logger quiet(nullptr);
  const sankhya::Solution want = sankhya::pdhg::solve_pdhg(model, options, quiet, nullptr);
  const sankhya::Solution got = sankhya::gpu::solve_pdhg_gpu(model, options, quiet, nullptr);
  std::printf("%s: status %s, %lld iterations, objective %.12g\n", label,
              sankhya::to_string(got.status), static_cast<long long>(got.iterations),
              got.objective);
  check(got.status == want.status, "status");
  check(got.iterations == want.iterations, "iterations");
  check(got.message == want.message, "message");
  check(got.algorithm == "pdhg-gpu", "algorithm");
  check(same(got.col_value, want.col_value), "col_value");
  check(same(got.col_dual, want.col_dual), "col_dual");
  check(same(got.row_dual, want.row_dual), "row_dual");
  check(same(got.row_activity, want.row_activity), "row_activity");
  check(same(got.objective, want.objective), "objective");
  check(same(got.dual_bound, want.dual_bound), "dual_bound");
  check(same(got.primal_infeasibility, want.primal_infeasibility), "primal_infeasibility");
  check(same(got.dual_infeasibility, want.dual_infeasibility), "dual_infeasibility");
  check(same(got.absolute_gap, want.absolute_gap), "absolute_gap");
  check(same(got.relative_gap, want.relative_gap), "relative_gap");
}

}  // namespace

int main() {
  const sankhya::Options options = make_options();
  sankhya::Logger quiet(nullptr);

  // No engine (the first call of the process, before the seam holds one): a numerical error
  // carrying the engine's message, and no CPU answer. The next call creates the engine.
  standin_fail_create(1);
  const sankhya::Solution d = sankhya::gpu::solve_pdhg_gpu(make_model(14, false), options, quiet, nullptr);
  standin_fail_create(0);
  check(d.status == sankhya::SolveStatus::kNumericalError, "no engine: status");
  check(d.message.find("stand-in") != std::string::npos, "no engine: the engine's message");
  check(d.iterations == 0, "no engine: no iterations");

  compare(make_model(11, false), "minimise");
  compare(make_model(12, true), "maximise");

  // A Model that fails validation never reaches the engine.
  sankhya::Model bad = make_model(13, false);
  bad.col_cost[3] = std::numeric_limits<double>::quiet_NaN();
  const sankhya::Solution b = sankhya::gpu::solve_pdhg_gpu(bad, options, quiet, nullptr);
  check(b.status == sankhya::SolveStatus::kModelError, "model error status");
  check(!b.message.empty(), "model error message");

  // An interrupt requested through SolveControl.
  sankhya::SolveControl control;
  control.interrupt();
  const sankhya::Solution i = sankhya::gpu::solve_pdhg_gpu(make_model(15, false), options, quiet, &control);
  check(i.status == sankhya::SolveStatus::kInterrupted, "interrupt status");

  // The iteration table goes through the Logger.
  std::FILE* log = std::tmpfile();
  sankhya::Logger logger(log);
  const sankhya::Solution l = sankhya::gpu::solve_pdhg_gpu(make_model(16, false), options, logger, nullptr);
  std::fflush(log);
  check(std::ftell(log) > 0, "iteration table written");
  std::fclose(log);
  check(l.status == sankhya::SolveStatus::kOptimal || l.status == sankhya::SolveStatus::kFeasible,
        "logged solve status");

  // Concurrent callers: every thread's answers must be its own Model's.
  {
    constexpr int kThreads = 4, kRounds = 3;
    std::vector<sankhya::Model> models;
    std::vector<sankhya::Solution> wants;
    for (int k = 0; k < kThreads; ++k) {
      models.push_back(make_model(30 + k, k % 2 == 1));
      wants.push_back(sankhya::pdhg::solve_pdhg(models.back(), options, quiet, nullptr));
    }
    std::vector<int> wrong(kThreads, 0);
    std::vector<std::thread> threads;
    for (int k = 0; k < kThreads; ++k) {
      threads.emplace_back([&, k] {
        sankhya::Logger own(nullptr);
        for (int r = 0; r < kRounds; ++r) {
          const sankhya::Solution got =
              sankhya::gpu::solve_pdhg_gpu(models[k], options, own, nullptr);
          const sankhya::Solution& want = wants[k];
          if (got.status != want.status || got.iterations != want.iterations ||
              !same(got.col_value, want.col_value) || !same(got.row_dual, want.row_dual) ||
              !same(got.objective, want.objective)) {
            ++wrong[k];
          }
        }
      });
    }
    for (auto& t : threads) t.join();
    for (int k = 0; k < kThreads; ++k) {
      check(wrong[k] == 0, "concurrent callers get their own answers");
    }
  }

  // The profile: the same restart counter as the CPU engine, and the GPU phases.
  {
    const sankhya::Model model = make_model(17, false);
    sankhya::Options o = make_options();
    o.set_bool("pdhg_stop_at_request", false);
    o.set_double("pdhg_tolerance", 1e-8);
    sankhya::Profiler cpu_profile(sankhya::ProfileMode::kBasic);
    sankhya::Profiler gpu_profile(sankhya::ProfileMode::kBasic);
    sankhya::Logger cpu_log(nullptr), gpu_log(nullptr);
    cpu_log.set_profiler(&cpu_profile);
    gpu_log.set_profiler(&gpu_profile);
    const sankhya::Solution c = sankhya::pdhg::solve_pdhg(model, o, cpu_log, nullptr);
    const sankhya::Solution g = sankhya::gpu::solve_pdhg_gpu(model, o, gpu_log, nullptr);
    auto counter = [](const sankhya::Profiler& p, const char* name) -> long long {
      for (const auto& k : p.counters()) {
        if (k.name == name) return k.value;
      }
      return -1;
    };
    const long long restarts = counter(cpu_profile, "pdhg restarts");
    check(restarts > 0, "profile: the CPU engine restarted");
    check(counter(gpu_profile, "pdhg restarts") == restarts, "profile: same restart count");
    bool phases = false;
    for (const auto& r : gpu_profile.regions()) {
      if (r.name == "pdhg iterations (gpu)" && r.calls == g.iterations) phases = true;
    }
    check(phases, "profile: the GPU iterations region");
    check(g.iterations == c.iterations, "profile: same solve");
  }

  if (g_failures != 0) {
    std::printf("%d failures\n", g_failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}

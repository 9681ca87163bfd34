// qp_seam_check.cpp -- convex QPs through the QP seam (seam/qp_gpu.cpp).
//
// `qp_seam_check standin [demo.mps ...]` is linked with the reference's core and the C-ABI
// stand-in (seam_standin.cpp, the reference's solve_convex_qp behind the engine's calls);
// `qp_seam_check gpu [demo.mps ...]` with the engine's real library. Every QP is solved by the
// seam and by the reference's own sankhya::qp::solve_convex_qp. The QPs: the convex instances
// of the reference's tests/unit/test_qp.cpp, seeded random convex QPs (both senses, with and
// without rows), the demo QPs given on the command line (read by the reference's reader), and
// the two non-convex instances of test_qp.cpp. Checks:
//   both modes: a non-convex QP is kModelError with the reference's message, word for word;
//   the iteration limit (777) and a zero time limit stop as the reference does, with its
//   messages; a raised interrupt is kInterrupted with the reference's message; the Solution
//   says "qp-condat-vu-gpu".
//   standin: every other Solution equals the reference's bit for bit (status, iterations,
//   objective, dual bound, the three vectors); an engine that cannot be created is
//   kNumericalError.
//   gpu: the same status and iteration count, the point and duals within 1e-8 of the
//   reference's scale and the objective within 1e-9 relative.
// Prints OK when every check passed.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "../../sih-26_gb300/seam/qp_gpu.hpp"
#include "sankhya/io.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/qp.hpp"
#include "sankhya/solve_control.hpp"
#include "sankhya/tolerances.hpp"

extern "C" {
void standin_fail_create(int fail) __attribute__((weak));
}

namespace {

using sankhya::kInfinity;

int g_failures = 0;

void check(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what.c_str());
    ++g_failures;
  }
}

bool same_bits(const std::vector<double>& a, const std::vector<double>& b) {
  return a.size() == b.size() &&
         (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(double)) == 0);
}

bool same_bits(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }

double scale_of(const std::vector<double>& v) {
  double s = 1.0;
  for (double x : v) s = std::max(s, std::fabs(x));
  return s;
}

bool near(const std::vector<double>& a, const std::vector<double>& b, double tol) {
  if (a.size() != b.size()) return false;
  const double s = scale_of(b);
  for (std::size_t k = 0; k < a.size(); ++k) {
    if (!(std::fabs(a[k] - b[k]) <= tol * s)) return false;
  }
  return true;
}

// make_qp of tests/unit/test_qp.cpp:34-68.
sankhya::Model make_qp(const std::vector<double>& cost, const std::vector<double>& lower,
                       const std::vector<double>& upper,
                       const std::vector<std::tuple<int, int, double>>& hessian,
                       const std::vector<std::vector<double>>& rows = {},
                       const std::vector<double>& row_lower = {},
                       const std::vector<double>& row_upper = {}) {
  sankhya::Model model;
  const int n = static_cast<int>(cost.size()), m = static_cast<int>(rows.size());
  model.col_cost = cost;
  model.col_lower = lower;
  model.col_upper = upper;
  model.col_type.assign(cost.size(), sankhya::VarType::kContinuous);
  model.row_lower = row_lower;
  model.row_upper = row_upper;
  model.matrix.reset(m, n);
  for (int i = 0; i < m; ++i) {
    for (int j = 0; j < n; ++j) {
      if (rows[i][j] != 0.0) model.matrix.add_entry(i, j, rows[i][j]);
    }
  }
  model.matrix.finalize();
  model.hessian.reset(n, n);
  for (const auto& [i, j, v] : hessian) model.hessian.add_entry(i, j, v);
  model.hessian.finalize();
  return model;
}

// A seeded convex QP: `per_column` N(0, 1) entries per column, rows around A x0 (a third of
// them equalities), columns in [-5, 5], a banded Hessian with a dominant diagonal.
sankhya::Model random_qp(unsigned seed, int m, int n, bool maximise) {
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> normal(0.0, 1.0);
  std::uniform_real_distribution<double> unit(0.0, 1.0);
  std::uniform_int_distribution<int> row_of(0, std::max(0, m - 1));
  sankhya::Model model;
  model.matrix.reset(m, n);
  std::vector<double> x0(n), ax(m, 0.0);
  for (int j = 0; j < n; ++j) {
    x0[j] = -2.0 + 4.0 * unit(rng);
    std::vector<int> used;
    for (int t = 0; t < 4 && m > 0; ++t) {
      const int r = row_of(rng);
      bool seen = false;
      for (int u : used) seen = seen || u == r;
      if (seen) continue;
      used.push_back(r);
      const double a = normal(rng);
      model.matrix.add_entry(r, j, a);
      ax[r] += a * x0[j];
    }
  }
  model.matrix.finalize();
  model.col_lower.assign(n, -5.0);
  model.col_upper.assign(n, 5.0);
  model.col_type.assign(n, sankhya::VarType::kContinuous);
  for (int j = 0; j < n; ++j) {
    if (j % 4 == 1) model.col_lower[j] = -kInfinity;
    if (j % 4 == 2) model.col_upper[j] = kInfinity;
    model.col_cost.push_back(normal(rng));
  }
  for (int i = 0; i < m; ++i) {
    const bool eq = i % 3 == 0;
    model.row_lower.push_back(eq ? ax[i] : ax[i] - 0.1 - unit(rng));
    model.row_upper.push_back(eq ? ax[i] : (i % 3 == 1 ? kInfinity : ax[i] + 0.1 + unit(rng)));
  }
  model.hessian.reset(n, n);
  std::vector<double> off(n, 0.0);
  std::vector<std::tuple<int, int, double>> lower;
  for (int j = 0; j + 1 < n; ++j) {
    const double v = 0.3 * normal(rng);
    lower.push_back({j + 1, j, v});
    off[j] += std::fabs(v);
    off[j + 1] += std::fabs(v);
  }
  for (int j = 0; j < n; ++j) lower.push_back({j, j, off[j] + 0.2 + unit(rng)});
  const double sign = maximise ? -1.0 : 1.0;
  for (const auto& [i, j, v] : lower) model.hessian.add_entry(i, j, sign * v);
  model.hessian.finalize();
  if (maximise) {
    model.sense = sankhya::ObjSense::kMaximize;
    for (double& c : model.col_cost) c = -c;
  }
  return model;
}

sankhya::Options qp_options(double tolerance) {
  sankhya::Options o;
  o.set_bool("log_to_console", false);
  o.set_double("qp_tolerance", tolerance);
  o.set_int("iteration_limit", 500000);
  return o;
}

// Everything before the elapsed seconds of a ResourceLimits::describe message.
std::string before_seconds(const std::string& message) {
  const std::size_t at = message.rfind(", ");
  return at == std::string::npos ? message : message.substr(0, at);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("usage: qp_seam_check standin|gpu [demo.mps ...]\n");
    return 2;
  }
  const bool standin = std::strcmp(argv[1], "standin") == 0;
  sankhya::Logger quiet(nullptr);

  std::vector<std::pair<std::string, sankhya::Model>> convex = {
      {"separable", make_qp({-2.0, -8.0}, {0, 0}, {kInfinity, kInfinity},
                            {{0, 0, 2.0}, {1, 1, 4.0}})},
      {"bound_cuts_off", make_qp({-2.0, -8.0}, {0, 0}, {0.25, kInfinity},
                                 {{0, 0, 2.0}, {1, 1, 4.0}})},
      {"coupling_row", make_qp({0.0, 0.0}, {0, 0}, {kInfinity, kInfinity},
                               {{0, 0, 1.0}, {1, 1, 1.0}}, {{1.0, 1.0}}, {2.0}, {2.0})},
      {"off_diagonal_twice", make_qp({-4.0, -4.0}, {0, 0}, {kInfinity, kInfinity},
                                     {{0, 0, 2.0}, {1, 0, 1.0}, {1, 1, 2.0}})},
      {"singular_semidefinite", make_qp({-2.0, -2.0}, {0, 0}, {10.0, 10.0},
                                        {{0, 0, 1.0}, {1, 0, 1.0}, {1, 1, 1.0}})},
      {"random_min", random_qp(11, 60, 120, false)},
      {"random_max", random_qp(12, 80, 150, true)},
      {"random_no_rows", random_qp(13, 0, 90, false)},
  };
  {
    sankhya::Model max1 = make_qp({2.0}, {0}, {kInfinity}, {{0, 0, -1.0}});
    max1.sense = sankhya::ObjSense::kMaximize;
    convex.push_back({"maximisation", max1});
  }
  for (int a = 2; a < argc; ++a) {
    sankhya::Model demo;
    const sankhya::io::ReadResult read = sankhya::io::read_model(argv[a], &demo);
    check(read.ok, std::string("read ") + argv[a]);
    if (read.ok) convex.push_back({argv[a], demo});
  }

  if (standin) {
    standin_fail_create(1);
    const sankhya::Solution s =
        sankhya::gpu::solve_convex_qp_gpu(convex[0].second, qp_options(1e-10), quiet);
    check(s.status == sankhya::SolveStatus::kNumericalError &&
              s.message.find("unavailable") != std::string::npos,
          "no engine: kNumericalError (" + s.message + ")");
    standin_fail_create(0);
  }

  for (const auto& [name, model] : convex) {
    const sankhya::Options o = qp_options(name.rfind("random", 0) == 0 ? 1e-8 : 1e-10);
    const sankhya::Solution ref = sankhya::qp::solve_convex_qp(model, o, quiet, nullptr);
    const sankhya::Solution got = sankhya::gpu::solve_convex_qp_gpu(model, o, quiet, nullptr);
    const std::string what = name + " (" + sankhya::to_string(got.status) + " vs " +
                             sankhya::to_string(ref.status) + ", " +
                             std::to_string(got.iterations) + " vs " +
                             std::to_string(ref.iterations) + " iterations)";
    check(got.algorithm == "qp-condat-vu-gpu", what + ": algorithm");
    check(ref.status == sankhya::SolveStatus::kOptimal, what + ": the reference solves it");
    check(got.status == ref.status && got.iterations == ref.iterations, what + ": status");
    if (standin) {
      check(same_bits(got.objective, ref.objective) && same_bits(got.dual_bound, ref.dual_bound) &&
                same_bits(got.col_value, ref.col_value) && same_bits(got.col_dual, ref.col_dual) &&
                same_bits(got.row_dual, ref.row_dual) && got.message == ref.message,
            what + ": the reference's Solution bit for bit");
    } else {
      check(near(got.col_value, ref.col_value, 1e-8) && near(got.col_dual, ref.col_dual, 1e-8) &&
                near(got.row_dual, ref.row_dual, 1e-8),
            what + ": the point and duals within 1e-8");
      check(std::fabs(got.objective - ref.objective) <= 1e-9 * std::max(1.0, std::fabs(ref.objective)),
            what + ": objective within 1e-9");
    }
    std::printf("%s: %s, %lld iterations, objective %.12g\n", name.c_str(),
                sankhya::to_string(got.status), static_cast<long long>(got.iterations),
                got.objective);
  }

  // The refusals: the reference's own convexity test and its message, word for word.
  const std::vector<std::pair<std::string, sankhya::Model>> nonconvex = {
      {"negative_curvature", make_qp({0.0, 0.0}, {-kInfinity, -kInfinity},
                                     {kInfinity, kInfinity}, {{0, 0, 1.0}, {1, 1, -1.0}})},
      {"hidden_off_diagonal", make_qp({0.0, 0.0}, {-kInfinity, -kInfinity},
                                      {kInfinity, kInfinity},
                                      {{0, 0, 1.0}, {1, 0, 3.0}, {1, 1, 1.0}})},
  };
  for (const auto& [name, model] : nonconvex) {
    const sankhya::Options o = qp_options(1e-10);
    const sankhya::Solution ref = sankhya::qp::solve_convex_qp(model, o, quiet, nullptr);
    const sankhya::Solution got = sankhya::gpu::solve_convex_qp_gpu(model, o, quiet, nullptr);
    check(got.status == sankhya::SolveStatus::kModelError && got.message == ref.message &&
              got.message.find("not convex") != std::string::npos,
          name + ": refused with the reference's message (" + got.message + ")");
  }

  // Limits and the interrupt, on one random QP, at a tolerance no run meets (the residuals
  // stop near rounding level).
  const sankhya::Model& limited = convex[5].second;
  {
    sankhya::Options o = qp_options(1e-30);
    o.set_int("iteration_limit", 777);
    const sankhya::Solution ref = sankhya::qp::solve_convex_qp(limited, o, quiet, nullptr);
    const sankhya::Solution got = sankhya::gpu::solve_convex_qp_gpu(limited, o, quiet, nullptr);
    check(got.status == sankhya::SolveStatus::kIterationLimit && got.iterations == 777 &&
              ref.iterations == 777 && before_seconds(got.message) == before_seconds(ref.message),
          "iteration limit 777 (" + got.message + " | " + ref.message + ")");
  }
  {
    sankhya::Options o = qp_options(1e-30);
    o.set_double("time_limit", 0.0);
    const sankhya::Solution ref = sankhya::qp::solve_convex_qp(limited, o, quiet, nullptr);
    const sankhya::Solution got = sankhya::gpu::solve_convex_qp_gpu(limited, o, quiet, nullptr);
    const std::string head = "stopped at the time limit of 0s after ";
    const std::string tail = ", 0 iterations, 0 nodes";
    const auto shaped = [&](const std::string& m) {
      return m.rfind(head, 0) == 0 && m.size() > tail.size() &&
             m.compare(m.size() - tail.size(), tail.size(), tail) == 0;
    };
    check(got.status == sankhya::SolveStatus::kTimeLimit && got.iterations == 0 &&
              ref.status == got.status && shaped(got.message) && shaped(ref.message),
          "time limit 0 (" + got.message + " | " + ref.message + ")");
    check(got.dual_bound == -kInfinity, "an unfinished run claims no bound");
  }
  {
    sankhya::SolveControl control;
    control.interrupt();
    const sankhya::Solution got =
        sankhya::gpu::solve_convex_qp_gpu(limited, qp_options(1e-30), quiet, &control);
    check(got.status == sankhya::SolveStatus::kInterrupted &&
              got.message.rfind("stopped by user interrupt after ", 0) == 0,
          "interrupt (" + got.message + ")");
  }
  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}

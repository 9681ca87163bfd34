// gradients_check.cpp -- the gradient surface at the seam (seam/lp_gradients.cpp) on the GPU.
//
// Linked with the reference's core, the seam and the engine's real library. A planted LP with
// a unique, nondegenerate optimum is built here: m equality rows, 2m columns in [0, 10]; the
// first m columns are basic at x0 in [1, 9], each with a heavy entry in its own row, the rest
// sit at 0 or 10; y0 ~ N(0, 1) and c = A'y0 + z with z = 0 on the basic columns, z > 0 at the
// lower bound and z < 0 at the upper. For the loss L = f* the gradients are known exactly:
// dL/dc = x0, dL/db = y0 (the row's multiplier), dL/d(bound) = z on the nonbasic columns'
// active bounds and 0 elsewhere. The maximisation of -c'x over the same rows has the same
// optimum: there dL/dc = x0 again and dL/db = -y0 (its reported multiplier). Each must hold to
// 1e-8 relative, and the written gradient file must hold one line per column and per row.
// Prints OK when every check passed.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "../../sih-26_gb300/seam/lp_gradients.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"

namespace {

int g_failures = 0;

void check(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what.c_str());
    ++g_failures;
  }
}

bool close(const std::vector<double>& a, const std::vector<double>& b, double tol) {
  if (a.size() != b.size()) return false;
  for (std::size_t k = 0; k < a.size(); ++k) {
    if (std::fabs(a[k] - b[k]) > tol * std::max(1.0, std::fabs(b[k]))) return false;
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string out_path = argc > 1 ? argv[1] : "gradients.txt";
  const int m = 60, n = 2 * m;
  std::mt19937_64 rng(2026);
  std::uniform_real_distribution<double> unit(0.0, 1.0);
  std::normal_distribution<double> normal(0.0, 1.0);
  std::uniform_int_distribution<int> row_of(0, m - 1);

  sankhya::Model model;
  model.sense = sankhya::ObjSense::kMinimize;
  model.matrix.reset(m, n);
  std::vector<double> x0(n), y0(m), z(n, 0.0);
  std::vector<std::vector<std::pair<int, double>>> cols(n);
  for (int j = 0; j < n; ++j) {
    if (j < m) cols[j].push_back({j, 5.0 + unit(rng)});
    while (cols[j].size() < 3) {
      const int r = row_of(rng);
      bool seen = false;
      for (const auto& e : cols[j]) seen = seen || e.first == r;
      if (!seen) cols[j].push_back({r, normal(rng)});
    }
    for (const auto& e : cols[j]) model.matrix.add_entry(e.first, j, e.second);
    x0[j] = j < m ? 1.0 + 8.0 * unit(rng) : (j % 2 == 0 ? 0.0 : 10.0);
  }
  model.matrix.finalize(0.0);
  for (int i = 0; i < m; ++i) y0[i] = normal(rng);
  model.col_lower.assign(n, 0.0);
  model.col_upper.assign(n, 10.0);
  model.col_type.assign(n, sankhya::VarType::kContinuous);
  model.col_cost.assign(n, 0.0);
  std::vector<double> b(m, 0.0);
  for (int j = 0; j < n; ++j) {
    double aty = 0.0;
    for (const auto& e : cols[j]) {
      b[e.first] += e.second * x0[j];
      aty += e.second * y0[e.first];
    }
    if (j >= m) z[j] = (j % 2 == 0 ? 1.0 : -1.0) * (0.5 + unit(rng));
    model.col_cost[j] = aty + z[j];
  }
  model.row_lower = b;
  model.row_upper = b;

  sankhya::Options options;
  options.set_bool("log_to_console", false);
  options.set_double("pdhg_tolerance", 1e-7);
  options.set_int("iteration_limit", 1000000);
  sankhya::Logger quiet(nullptr);
  sankhya::gpu::LossGradient loss;
  loss.by_f = 1.0;

  std::vector<double> dl(n, 0.0), du(n, 0.0);
  for (int j = m; j < n; ++j) (x0[j] <= 0.0 ? dl : du)[j] = z[j];

  for (const bool maximise : {false, true}) {
    sankhya::Model lp = model;
    if (maximise) {
      lp.sense = sankhya::ObjSense::kMaximize;
      for (double& c : lp.col_cost) c = -c;
    }
    const auto [sol, g] = sankhya::gpu::solve_pdhg_gpu_with_gradients(lp, options, quiet, loss);
    const std::string tag = maximise ? "maximise" : "minimise";
    std::printf("%s: %s, %lld iterations; %s\n", tag.c_str(), sankhya::to_string(sol.status),
                static_cast<long long>(sol.iterations), g.message.c_str());
    check(g.status == 0, tag + ": gradients hold (" + g.message + ")");
    check(close(sol.col_value, x0, 1e-8), tag + ": the polished point is the planted vertex");
    check(close(g.cost, x0, 1e-8), tag + ": dL/dc = x*");
    std::vector<double> db(m);
    for (int i = 0; i < m; ++i) db[i] = g.row_lower[i] + g.row_upper[i];
    std::vector<double> want_y = y0;
    if (maximise) {
      for (double& v : want_y) v = -v;
    }
    check(close(db, want_y, 1e-8), tag + ": dL/db = y*");
    // The bound gradients of f* are the reduced costs of the active bounds, in the LP's own
    // sense (a maximisation's reduced costs are those of its negated minimisation, negated).
    std::vector<double> want_l = dl, want_u = du;
    if (maximise) {
      for (double& v : want_l) v = -v;
      for (double& v : want_u) v = -v;
    }
    check(close(g.col_lower, want_l, 1e-8) && close(g.col_upper, want_u, 1e-8),
          tag + ": dL/d(bound) = the active bounds' reduced costs");
    if (!maximise) {
      std::string error;
      check(sankhya::gpu::write_gradients(out_path, lp, g, &error), "write_gradients: " + error);
      std::ifstream in(out_path);
      int lines = 0, col_lines = 0, row_lines = 0;
      for (std::string line; std::getline(in, line);) {
        ++lines;
        col_lines += line.rfind("col ", 0) == 0;
        row_lines += line.rfind("row ", 0) == 0;
      }
      check(col_lines == n && row_lines == m && lines == n + m + 1,
            "the gradient file has one line per column and per row");
    }
  }
  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}

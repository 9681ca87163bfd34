// node_batch_check.cpp -- node relaxations through the node-batch seam (seam/node_batch.cpp).
//
// `node_batch_check model.mps standin` is linked with the reference's core and the C-ABI
// stand-in (seam_standin.cpp, one reference solve_pdhg per LP); `node_batch_check model.mps
// gpu` with the engine's real library. Both read the model with the reference's reader, solve
// its root with the reference's CPU PDHG, and branch on its fractional columns the way a
// branch-and-bound search does: node 2t tightens column j_t to [l, floor(x_j)], node 2t + 1 to
// [ceil(x_j), u]. One more node fixes the columns of one row (with a finite upper side) so that
// the row cannot hold: the row's unit vector is its Farkas certificate. Checks:
//   standin: every branching node's Solution equals the reference's solve_pdhg of that node
//   bit for bit (status, iterations, objective, the three vectors) and says "pdhg-gpu-batch";
//   the infeasible node, given its certificate, is kInfeasible with the host check's message;
//   a feasible node given the same direction as a would-be certificate is kNumericalError
//   (the host check refuses it); bounds of the wrong length make every node kModelError; a
//   batched engine that cannot be created makes every node kNumericalError.
//   gpu: every branching node that the reference solves to optimal or feasible comes back
//   optimal or feasible with the objective within 1e-6 relative; the infeasible node comes
//   back kInfeasible with a certificate that checked on the host, or unsolved at the
//   iteration limit (see below), never solved.
// Prints OK when every check passed.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../sih-26_gb300/seam/node_batch.hpp"
#include "sankhya/io.hpp"
#include "sankhya/model.hpp"
#include "sankhya/options.hpp"
#include "sankhya/pdhg.hpp"

extern "C" {
void standin_fail_create(int fail) __attribute__((weak));
void standin_batch_mark_infeasible(int index, const double* ray, int rows) __attribute__((weak));
void standin_batch_clear_marks(void) __attribute__((weak));
}

namespace {

int g_failures = 0;

void check(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL: %s\n", what.c_str());
    ++g_failures;
  }
}

bool same(const std::vector<double>& a, const std::vector<double>& b) {
  return a.size() == b.size() &&
         (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(double)) == 0);
}

bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }

sankhya::Options node_options() {
  sankhya::Options o;
  o.set_bool("log_to_console", false);
  o.set_double("pdhg_tolerance", 1e-6);
  o.set_int("iteration_limit", 200000);
  return o;
}

bool solved(sankhya::SolveStatus s) {
  return s == sankhya::SolveStatus::kOptimal || s == sankhya::SolveStatus::kFeasible;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::printf("usage: node_batch_check model.mps standin|gpu\n");
    return 2;
  }
  const bool standin = std::strcmp(argv[2], "standin") == 0;
  sankhya::Model model;
  const sankhya::io::ReadResult read = sankhya::io::read_model(argv[1], &model);
  if (!read.ok) {
    std::printf("cannot read %s: %s\n", argv[1], read.error.c_str());
    return 2;
  }
  const sankhya::Options options = node_options();
  sankhya::Logger quiet(nullptr);
  const auto n = static_cast<std::size_t>(model.num_cols());
  const auto m = static_cast<std::size_t>(model.num_rows());

  // Branching nodes on the root's fractional columns.
  const sankhya::Solution root = sankhya::pdhg::solve_pdhg(model, options, quiet, nullptr);
  std::vector<sankhya::gpu::NodeBounds> nodes;
  for (std::size_t j = 0; j < n && nodes.size() < 12; ++j) {
    const double x = root.col_value[j];
    const double f = x - std::floor(x);
    if (f < 0.1 || f > 0.9) continue;
    sankhya::gpu::NodeBounds down{model.col_lower, model.col_upper};
    sankhya::gpu::NodeBounds up{model.col_lower, model.col_upper};
    down.col_upper[j] = std::floor(x);
    up.col_lower[j] = std::ceil(x);
    if (down.col_upper[j] >= down.col_lower[j]) nodes.push_back(down);
    if (up.col_lower[j] <= up.col_upper[j]) nodes.push_back(up);
  }
  check(nodes.size() >= 4, "at least four branching nodes");
  const std::size_t branching = nodes.size();

  // The infeasible node: the columns of the first row with a finite upper side and a nonzero
  // entry are fixed at +-(1 + |ru| / |a_ij|), which puts that row's activity above ru.
  std::vector<std::vector<std::pair<std::size_t, double>>> row_entries(m);
  {
    const auto& starts = model.matrix.column_starts();
    const auto& rows = model.matrix.row_indices();
    const auto& values = model.matrix.values();
    for (std::size_t j = 0; j < n; ++j) {
      for (auto k = starts[j]; k < starts[j + 1]; ++k) {
        if (values[k] != 0.0) {
          row_entries[static_cast<std::size_t>(rows[k])].push_back({j, values[k]});
        }
      }
    }
  }
  std::size_t row = m;
  for (std::size_t i = 0; i < m && row == m; ++i) {
    if (sankhya::is_finite_bound(model.row_upper[i]) && !row_entries[i].empty()) row = i;
  }
  check(row < m, "a row with a finite upper side");
  sankhya::gpu::NodeBounds bad{model.col_lower, model.col_upper};
  std::vector<double> certificate(m, 0.0);
  if (row < m) {
    const double ru = model.row_upper[row];
    for (const auto& [j, a] : row_entries[row]) {
      const double v = (1.0 + std::fabs(ru)) / std::fabs(a) * (a > 0.0 ? 1.0 : -1.0);
      bad.col_lower[j] = v;
      bad.col_upper[j] = v;
    }
    certificate[row] = 1.0;
  }
  const std::size_t infeasible_node = nodes.size();
  nodes.push_back(bad);

  if (standin) {
    // No engine: every node is a numerical error with the engine's message.
    standin_fail_create(1);
    const auto failed = sankhya::gpu::solve_node_relaxations_gpu(model, nodes, options, quiet);
    for (const auto& s : failed) {
      check(s.status == sankhya::SolveStatus::kNumericalError &&
                s.message.find("unavailable") != std::string::npos,
            "no engine: kNumericalError (" + s.message + ")");
    }
    standin_fail_create(0);
    // The infeasible node carries its certificate; root-like node 0 a direction that proves
    // nothing.
    standin_batch_clear_marks();
    standin_batch_mark_infeasible(static_cast<int>(infeasible_node), certificate.data(),
                                  static_cast<int>(m));
    standin_batch_mark_infeasible(0, certificate.data(), static_cast<int>(m));
  }
  const auto got = sankhya::gpu::solve_node_relaxations_gpu(model, nodes, options, quiet);
  check(got.size() == nodes.size(), "one Solution per node");
  for (std::size_t k = 0; k < got.size() && k < nodes.size(); ++k) {
    const sankhya::Solution& s = got[k];
    check(s.algorithm == "pdhg-gpu-batch", "algorithm pdhg-gpu-batch");
    if (k == infeasible_node) {
      const bool proved = s.status == sankhya::SolveStatus::kInfeasible &&
                          s.message.find("checked on the host") != std::string::npos;
      // The engine's Farkas test takes the dual change over a restart period as the
      // direction, and a direction with any component that leans on an absent bound proves
      // nothing: on a model with one-sided rows and columns (afiro's) the noise in those
      // components keeps it from proving this node infeasible, and the node then ends at the
      // iteration limit. It must never come back as a solved node.
      check(standin ? proved : (proved || s.status == sankhya::SolveStatus::kIterationLimit),
            "the infeasible node is kInfeasible with a checked certificate" +
                std::string(standin ? "" : ", or unsolved") + " (" +
                std::string(sankhya::to_string(s.status)) + ": " + s.message + ")");
      std::printf("infeasible node: %s\n", sankhya::to_string(s.status));
      continue;
    }
    if (standin && k == 0) {
      check(s.status == sankhya::SolveStatus::kNumericalError,
            "a certificate that does not check is refused (" + s.message + ")");
      continue;
    }
    sankhya::Model node = model;
    node.col_lower = nodes[k].col_lower;
    node.col_upper = nodes[k].col_upper;
    const sankhya::Solution ref = sankhya::pdhg::solve_pdhg(node, options, quiet, nullptr);
    const std::string what = "node " + std::to_string(k) + " (" +
                             sankhya::to_string(s.status) + " vs " +
                             sankhya::to_string(ref.status) + ")";
    if (standin) {
      check(s.status == ref.status && s.iterations == ref.iterations &&
                same(s.objective, ref.objective) && same(s.col_value, ref.col_value) &&
                same(s.col_dual, ref.col_dual) && same(s.row_dual, ref.row_dual),
            what + ": the reference's solve_pdhg bit for bit");
    } else if (solved(ref.status)) {
      const double rel = std::fabs(s.objective - ref.objective) /
                         std::max(1.0, std::fabs(ref.objective));
      check(solved(s.status) && rel <= 1e-6,
            what + ": objective " + std::to_string(s.objective) + " vs " +
                std::to_string(ref.objective));
    }
    std::printf("node %zu: %s, %lld iterations, objective %.10g\n", k,
                sankhya::to_string(s.status), static_cast<long long>(s.iterations), s.objective);
  }
  if (standin) {
    std::vector<sankhya::gpu::NodeBounds> wrong = {nodes[0]};
    wrong[0].col_lower.pop_back();
    const auto refused = sankhya::gpu::solve_node_relaxations_gpu(model, wrong, options, quiet);
    check(refused.size() == 1 && refused[0].status == sankhya::SolveStatus::kModelError,
          "bounds of the wrong length: kModelError");
    standin_batch_clear_marks();
  }
  std::printf("%zu branching nodes and one infeasible node\n", branching);
  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}

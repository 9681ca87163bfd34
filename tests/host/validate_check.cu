// validate_check.cu -- the engine's model checks (sgb::validate_lp, run by
// sankhya_gb300_pdhg_load and sankhya_gb300_batch_load) on the CPU, against the rules of
// the reference's Model::validate (src/core/model.cpp:127-240).
//
// Built by tests/test_host_layout.py against the engine's objects; no CUDA call is made. A
// valid LP (with infinite bounds, an empty column and an empty row) must pass. Each defect
// Model::validate refuses must be SANKHYA_GB300_ERROR_MODEL: a matrix value that is NaN or
// infinite (:178), a NaN bound or a crossed bound on a column or a row (:210-224), a NaN
// cost (:214), a NaN objective offset (:228). So must the CSC defects that a frozen
// SparseMatrix cannot hold (an out-of-range or repeated row index, starts that do not begin
// at 0 or go backwards) and, by the engine's own rule, an infinite cost. Negative sizes are
// SANKHYA_GB300_ERROR_ARGUMENT.
#include <cmath>
#include <cstdio>
#include <limits>
#include <string>
#include <vector>

#include "engine.hpp"

using namespace sgb;

namespace {

int g_failures = 0;

struct Lp {
  int rows = 3, cols = 4;
  std::vector<int32_t> starts{0, 2, 3, 3, 5};  // column 2 is empty
  std::vector<int32_t> index{0, 1, 0, 0, 1};   // row 2 is empty
  std::vector<double> values{1.0, -2.0, 3.0, 0.5, 4.0};
  std::vector<double> cost{1.0, -1.0, 0.0, 2.0};
  std::vector<double> lower{0.0, -INFINITY, 0.0, -1e30};
  std::vector<double> upper{10.0, 5.0, INFINITY, 1e30};
  std::vector<double> row_lower{1.0, -INFINITY, 0.0};
  std::vector<double> row_upper{1.0, 3.0, INFINITY};
  double offset = 2.5;

  sankhya_gb300_lp view() const {
    sankhya_gb300_lp lp{};
    lp.rows = rows;
    lp.cols = cols;
    lp.col_starts = starts.data();
    lp.row_index = index.data();
    lp.values = values.data();
    lp.col_cost = cost.data();
    lp.col_lower = lower.data();
    lp.col_upper = upper.data();
    lp.row_lower = row_lower.data();
    lp.row_upper = row_upper.data();
    lp.sense = 1.0;
    lp.objective_offset = offset;
    return lp;
  }
};

int code_of(const Lp& lp) {
  try {
    validate_lp(lp.view());
  } catch (const EngineError& e) {
    return e.code;
  }
  return SANKHYA_GB300_OK;
}

template <typename Edit>
void expect(const char* what, int want, Edit edit) {
  Lp lp;
  edit(lp);
  const int got = code_of(lp);
  if (got != want) {
    std::printf("FAIL: %s: code %d, expected %d\n", what, got, want);
    ++g_failures;
  }
}

}  // namespace

int main() {
  const double nan = std::numeric_limits<double>::quiet_NaN();
  constexpr int kOk = SANKHYA_GB300_OK;
  constexpr int kModel = SANKHYA_GB300_ERROR_MODEL;
  constexpr int kArgument = SANKHYA_GB300_ERROR_ARGUMENT;

  expect("a valid LP", kOk, [](Lp&) {});
  expect("an explicit zero in the matrix", kOk, [](Lp& lp) { lp.values[1] = 0.0; });
  expect("equal bounds (a fixed column and an equality row)", kOk, [](Lp& lp) {
    lp.lower[0] = lp.upper[0] = 3.0;
  });
  expect("an empty LP", kOk, [](Lp& lp) {
    lp = Lp();
    lp.rows = lp.cols = 0;
    lp.starts = {0};
  });

  expect("a NaN matrix value", kModel, [=](Lp& lp) { lp.values[2] = nan; });
  expect("an infinite matrix value", kModel, [](Lp& lp) { lp.values[3] = -INFINITY; });
  expect("a NaN column bound", kModel, [=](Lp& lp) { lp.upper[1] = nan; });
  expect("a crossed column bound", kModel, [](Lp& lp) { lp.lower[0] = 11.0; });
  expect("a NaN row bound", kModel, [=](Lp& lp) { lp.row_lower[2] = nan; });
  expect("a crossed row bound", kModel, [](Lp& lp) { lp.row_lower[1] = 4.0; });
  expect("a NaN cost", kModel, [=](Lp& lp) { lp.cost[2] = nan; });
  expect("a NaN objective offset", kModel, [=](Lp& lp) { lp.offset = nan; });
  expect("an infinite cost (the engine's own rule)", kModel,
         [](Lp& lp) { lp.cost[0] = INFINITY; });
  expect("a row index out of range", kModel, [](Lp& lp) { lp.index[2] = 3; });
  expect("a negative row index", kModel, [](Lp& lp) { lp.index[2] = -1; });
  expect("a repeated row index in a column", kModel, [](Lp& lp) { lp.index[1] = 0; });
  expect("row indices descending in a column", kModel, [](Lp& lp) {
    lp.index[0] = 1;
    lp.index[1] = 0;
  });
  expect("column starts not from 0", kModel, [](Lp& lp) { lp.starts[0] = 1; });
  expect("column starts going backwards", kModel, [](Lp& lp) { lp.starts[2] = 1; });
  expect("negative sizes", kArgument, [](Lp& lp) { lp.rows = -1; });

  if (g_failures == 0) std::printf("OK\n");
  return g_failures == 0 ? 0 : 1;
}

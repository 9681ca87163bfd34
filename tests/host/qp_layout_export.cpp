// qp_layout_export.cpp -- the convex-QP engine's host layouts (sih-26_gb300/csrc/qp_layout.hpp,
// the functions QpEngine::load and QpEngine::layout call) behind a small C interface, so that
// tests/test_qp_layout.py can check them on the CPU against an independent numpy build. Test
// infrastructure only.
#include <cstring>

#include "qp_layout.hpp"

extern "C" {

// Sizes of the layout: nonzeros of A (by rows) and of the full symmetric Q.
void qp_layout_sizes(const sankhya_gb300_qp_problem* p, long long* row_nnz, long long* q_nnz) {
  sgb::QpHostLayout h;
  sgb::qp_build_layout(*p, &h);
  *row_nnz = static_cast<long long>(h.row_cols.size());
  *q_nnz = static_cast<long long>(h.q_cols.size());
}

void qp_layout_fill(const sankhya_gb300_qp_problem* p, int* row_starts, int* row_cols,
                    double* row_values, int* q_starts, int* q_cols, double* q_values,
                    int* col_len, int* row_len, double* cost, double* col_lower,
                    double* col_upper, double* row_lower, double* row_upper) {
  sgb::QpHostLayout h;
  sgb::qp_build_layout(*p, &h);
  const auto copy = [](auto* dst, const auto& src) {
    if (!src.empty()) std::memcpy(dst, src.data(), src.size() * sizeof(src[0]));
  };
  copy(row_starts, h.row_starts);
  copy(row_cols, h.row_cols);
  copy(row_values, h.row_values);
  copy(q_starts, h.q_starts);
  copy(q_cols, h.q_cols);
  copy(q_values, h.q_values);
  copy(col_len, h.col_len);
  copy(row_len, h.row_len);
  copy(cost, h.cost);
  copy(col_lower, h.col_lower);
  copy(col_upper, h.col_upper);
  copy(row_lower, h.row_lower);
  copy(row_upper, h.row_upper);
}

// The chunk table for `count` items of the given lengths: six ints per chunk (item, begin,
// end, first, count, slot) into `out` (room for `capacity` chunks). Returns the chunk count
// (or -1 when it does not fit); *nlong receives the long items' count.
int qp_layout_chunks(const int* len, int count, int lanes, int* out, int capacity, int* nlong) {
  std::vector<int> l(len, len + count);
  std::vector<sgb::QpChunk> chunks;
  sgb::qp_build_chunks(l, lanes, &chunks, nlong);
  if (static_cast<int>(chunks.size()) > capacity) return -1;
  for (std::size_t k = 0; k < chunks.size(); ++k) {
    const sgb::QpChunk& c = chunks[k];
    const int row[6] = {c.item, c.begin, c.end, c.first, c.count, c.slot};
    std::memcpy(out + 6 * k, row, sizeof(row));
  }
  return static_cast<int>(chunks.size());
}

int qp_layout_lanes(double mean) { return sgb::qp_auto_lanes(mean); }

}  // extern "C"

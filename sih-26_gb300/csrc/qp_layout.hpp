// qp_layout.hpp -- the host-side layouts of the convex-QP engine, with no CUDA in them: what
// QpEngine::load and QpEngine::layout build from a sankhya_gb300_qp_problem (qp.cu), kept
// apart so that the CPU tests can check them (tests/host/qp_layout_export.cpp).
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <utility>
#include <vector>

#include "sankhya_gb300.h"

namespace sgb {

// Entries a chunk of a long row or column holds at most, and the lanes past which an item is
// long: an item with more than kQpLongPerLane entries per lane goes to the chunked path.
constexpr int kQpChunk = 2048;
constexpr int kQpLongPerLane = 64;

// One chunk of a long row or column: entries [begin, end) of the item's entry sequence (for
// a column: the entries of row j of Q, then those of column j of A).
struct QpChunk {
  int item;
  int begin, end;
  int first;  // the item's first chunk (partials slot)
  int count;  // the item's chunk count
  int slot;   // the item's ticket and long-item slot
};

// What the kernels read, built on the host.
struct QpHostLayout {
  // A by rows: a counting-sort transpose in column order keeps each row's columns ascending.
  std::vector<int> row_starts, row_cols;
  std::vector<double> row_values;
  // sense Q by rows, both triangles: a stored entry (i, j) is Q_ij and, off the diagonal, Q_ji
  // (src/qp/qp_condat_vu.cpp:145-160); columns ascending inside each row.
  std::vector<int> q_starts, q_cols;
  std::vector<double> q_values;
  // Entries per column (its row of Q and its column of A) and per row.
  std::vector<int> col_len, row_len;
  // The cost times the sense, and every bound that is_finite_bound calls absent as an
  // infinity on its side (include/sankhya/types.hpp:88-96).
  std::vector<double> cost, col_lower, col_upper, row_lower, row_upper;
};

inline bool qp_finite_bound(double v) { return !(std::isinf(v) || std::fabs(v) >= 1e30); }

// Builds every array of QpHostLayout. The problem must have passed the engine's load checks.
inline void qp_build_layout(const sankhya_gb300_qp_problem& p, QpHostLayout* out) {
  const sankhya_gb300_lp& lp = p.lp;
  const int m = lp.rows, n = lp.cols;
  const long long nnz = lp.col_starts[n];
  const long long hz = p.hessian_starts != nullptr ? p.hessian_starts[n] : 0;
  const double sense = lp.sense < 0.0 ? -1.0 : 1.0;

  out->row_starts.assign(static_cast<size_t>(m) + 1, 0);
  std::vector<int>& rptr = out->row_starts;
  for (long long k = 0; k < nnz; ++k) ++rptr[static_cast<size_t>(lp.row_index[k]) + 1];
  for (int i = 0; i < m; ++i) rptr[i + 1] += rptr[i];
  std::vector<int> next(rptr.begin(), rptr.end() - 1);
  out->row_cols.assign(static_cast<size_t>(nnz), 0);
  out->row_values.assign(static_cast<size_t>(nnz), 0.0);
  for (int j = 0; j < n; ++j) {
    for (int k = lp.col_starts[j]; k < lp.col_starts[j + 1]; ++k) {
      const int slot = next[lp.row_index[k]]++;
      out->row_cols[slot] = j;
      out->row_values[slot] = lp.values[k];
    }
  }

  // Walking the stored columns in order puts each row's entries in ascending column order for
  // a lower triangle; any other input is sorted per row.
  out->q_starts.assign(static_cast<size_t>(n) + 1, 0);
  std::vector<int>& qptr = out->q_starts;
  for (int j = 0; j < n && hz > 0; ++j) {
    for (int k = p.hessian_starts[j]; k < p.hessian_starts[j + 1]; ++k) {
      const int i = p.hessian_index[k];
      ++qptr[static_cast<size_t>(i) + 1];
      if (i != j) ++qptr[static_cast<size_t>(j) + 1];
    }
  }
  for (int j = 0; j < n; ++j) qptr[j + 1] += qptr[j];
  const long long qz = qptr[n];
  std::vector<int> qnext(qptr.begin(), qptr.end() - 1);
  std::vector<int>& qidx = out->q_cols;
  std::vector<double>& qval = out->q_values;
  qidx.assign(static_cast<size_t>(qz), 0);
  qval.assign(static_cast<size_t>(qz), 0.0);
  for (int j = 0; j < n && hz > 0; ++j) {
    for (int k = p.hessian_starts[j]; k < p.hessian_starts[j + 1]; ++k) {
      const int i = p.hessian_index[k];
      const double v = sense * p.hessian_values[k];
      int slot = qnext[i]++;
      qidx[slot] = j;
      qval[slot] = v;
      if (i != j) {
        slot = qnext[j]++;
        qidx[slot] = i;
        qval[slot] = v;
      }
    }
  }
  for (int r = 0; r < n; ++r) {
    const int b = qptr[r], e = qptr[r + 1];
    bool sorted = true;
    for (int k = b + 1; k < e && sorted; ++k) sorted = qidx[k - 1] <= qidx[k];
    if (sorted) continue;
    std::vector<std::pair<int, double>> row;
    for (int k = b; k < e; ++k) row.push_back({qidx[k], qval[k]});
    std::stable_sort(row.begin(), row.end(),
                     [](const auto& a, const auto& c) { return a.first < c.first; });
    for (int k = b; k < e; ++k) {
      qidx[k] = row[k - b].first;
      qval[k] = row[k - b].second;
    }
  }

  out->col_len.assign(static_cast<size_t>(n), 0);
  out->row_len.assign(static_cast<size_t>(m), 0);
  for (int j = 0; j < n; ++j) {
    out->col_len[j] = (qptr[j + 1] - qptr[j]) + (lp.col_starts[j + 1] - lp.col_starts[j]);
  }
  for (int i = 0; i < m; ++i) out->row_len[i] = rptr[i + 1] - rptr[i];

  constexpr double kInf = std::numeric_limits<double>::infinity();
  out->cost.resize(static_cast<size_t>(n));
  out->col_lower.resize(static_cast<size_t>(n));
  out->col_upper.resize(static_cast<size_t>(n));
  out->row_lower.resize(static_cast<size_t>(m));
  out->row_upper.resize(static_cast<size_t>(m));
  for (int j = 0; j < n; ++j) {
    out->cost[j] = sense * lp.col_cost[j];
    out->col_lower[j] = qp_finite_bound(lp.col_lower[j]) ? lp.col_lower[j] : -kInf;
    out->col_upper[j] = qp_finite_bound(lp.col_upper[j]) ? lp.col_upper[j] : kInf;
  }
  for (int i = 0; i < m; ++i) {
    out->row_lower[i] = qp_finite_bound(lp.row_lower[i]) ? lp.row_lower[i] : -kInf;
    out->row_upper[i] = qp_finite_bound(lp.row_upper[i]) ? lp.row_upper[i] : kInf;
  }
}

// The chunks of the items longer than kQpLongPerLane * lanes entries, in item order; *nlong
// receives the number of such items (their slots are 0 .. *nlong - 1 in item order).
inline void qp_build_chunks(const std::vector<int>& len, int lanes, std::vector<QpChunk>* out,
                            int* nlong) {
  out->clear();
  *nlong = 0;
  for (int item = 0; item < static_cast<int>(len.size()); ++item) {
    const int l = len[item];
    if (l <= kQpLongPerLane * lanes) continue;
    const int count = (l + kQpChunk - 1) / kQpChunk;
    const int first = static_cast<int>(out->size());
    for (int c = 0; c < count; ++c) {
      out->push_back(QpChunk{item, c * kQpChunk, std::min(l, (c + 1) * kQpChunk), first, count,
                             *nlong});
    }
    ++*nlong;
  }
}

// Lanes per item from the mean entries per item: the smallest power of two that leaves each
// lane at most 32 entries of a typical item. The passes wait on memory and on the FP64 pipe,
// where a lane that sits out the epilogue costs as much as a working one, so few lanes win:
// on the 1M x 2M QP (15 entries per column, 20 per row) one lane per column and per row runs
// 2.4 and 2.6 times faster than four and eight. Items longer than kQpLongPerLane lanes' worth
// go to the chunked path whatever the lanes.
inline int qp_auto_lanes(double mean) {
  int g = 1;
  while (g < 32 && 32.0 * g < mean) g *= 2;
  return g;
}

}  // namespace sgb

// qp_engine.hpp -- host side of the convex-QP engine (one QP, one device).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "engine.hpp"
#include "qp.cuh"
#include "sankhya_gb300.h"

namespace sgb {

class QpEngine {
 public:
  explicit QpEngine(int device);
  ~QpEngine();
  QpEngine(const QpEngine&) = delete;
  QpEngine& operator=(const QpEngine&) = delete;

  void load(const sankhya_gb300_qp_problem& p);
  void solve(const sankhya_gb300_qp_params& p, sankhya_gb300_qp_result* r);
  void solution(double* col_value, double* col_dual, double* row_dual);
  void time_kernels(int reps, double* ms);

 private:
  void require_loaded() const;
  // The chunk layouts of the long rows and columns for the given lanes (an item longer than
  // 64 lanes' worth of entries is chunked), and the device arrays that go with them.
  void layout(int col_lanes, int row_lanes);
  QpDev dev() const;
  double spectral_norm(unsigned seed);
  double hessian_norm(unsigned seed);
  double dot(const double* a, const double* b, int n);
  void build_graph(int periods);
  void destroy_graph();

  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  bool loaded_ = false;
  bool solved_ = false;

  int m_ = 0, n_ = 0;
  long long nnz_a_ = 0, nnz_q_ = 0, nnz_q_stored_ = 0;
  double sense_ = 1.0, offset_ = 0.0;
  std::vector<int> col_len_, row_len_;  // entries per column (Q row + A column) and per row

  DeviceArray<int> a_cs_, a_ri_, a_rs_, a_ci_, q_rs_, q_ci_;
  DeviceArray<double> a_cv_, a_rv_, q_v_, cost_, col_lower_, col_upper_, row_lower_,
      row_upper_;
  DeviceArray<double> x0_, x1_, xbar_, y_, col_dual_, row_dual_, vec_n_, vec_m_, dot_part_,
      dot_out_;

  // Layout for the current lanes.
  int col_lanes_ = 0, row_lanes_ = 0;
  int stage_ = 0;
  int col_short_blocks_ = 0, row_short_blocks_ = 0;
  int ncol_chunks_ = 0, nrow_chunks_ = 0, nlong_cols_ = 0, nlong_rows_ = 0;
  DeviceArray<QpChunk> col_chunks_, row_chunks_;
  DeviceArray<double2> col_part_, row_part_;
  DeviceArray<unsigned int> col_tickets_, row_tickets_;
  DeviceArray<double> long_col_obj_, obj_part_;

  DeviceArray<QpCtl> ctl_;
  DeviceArray<QpHist> hist_;
  QpCtl* ctl_host_ = nullptr;   // page-locked
  QpHist* hist_host_ = nullptr; // page-locked, kQpMaxPeriods entries
  long long final_iterations_ = 0;

  cudaGraphExec_t graph_ = nullptr;
  int graph_periods_ = 0, graph_col_lanes_ = 0, graph_row_lanes_ = 0, graph_stage_ = -1;
  long long graph_nodes_ = 0;
};

}  // namespace sgb

// batch_engine.hpp -- the host side of the batched solve (batch.cuh): packing many LPs, one
// copy per distinct matrix, and the two persistent launches.
#pragma once

#include <vector>

#include "batch.cuh"
#include "engine.hpp"
#include "sankhya_gb300.h"

namespace sgb {

class BatchEngine {
 public:
  explicit BatchEngine(int device);
  ~BatchEngine();

  void load(int count, const sankhya_gb300_lp* lps);
  void solve(const sankhya_gb300_params& params, sankhya_gb300_batch_item* items,
             double* device_seconds);
  void solution(int index, double* col_value, double* col_dual, double* row_dual);
  int count() const { return count_; }
  int distinct_matrices() const { return static_cast<int>(mats_.size()); }

 private:
  void require_loaded() const;

  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t timing_[2] = {nullptr, nullptr};
  int num_sms_ = 0;
  int count_ = 0;
  bool solved_ = false;
  std::vector<BatchMatrix> mats_;
  std::vector<BatchInstance> inst_;

  DeviceArray<BatchMatrix> d_mats_, d_mats_out_;
  DeviceArray<BatchInstance> d_inst_;
  DeviceArray<int> d_order_;
  DeviceArray<unsigned int> d_queue_;
  DeviceArray<int> csc_ptr_, csc_idx_, csr_ptr_, csr_idx_;
  DeviceArray<double> csc_raw_, csr_raw_, csc_s_, csr_s_;
  DeviceArray<double> dr_, dc_, row_acc_, col_acc_, power_v_, power_av_;
  DeviceArray<double> cost_, col_cost_, l_, u_, rl_, ru_;
  DeviceArray<double> cs_, ls_, us_, rls_, rus_;
  DeviceArray<double> x0_, x1_, x_sum_, x_rst_, xu0_, xu1_, best_x_, reduced_;
  DeviceArray<double2> xd_;
  DeviceArray<double> y0_, y1_, y_sum_, y_rst_, yu0_, yu1_, best_y_, ray_;
  DeviceArray<BatchOutcome> outcome_;
  long long total_n_ = 0, total_m_ = 0, mat_n_ = 0, mat_m_ = 0;
};

}  // namespace sgb

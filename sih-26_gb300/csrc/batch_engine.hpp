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
  // The last direction LP `index` tested as a Farkas certificate (m entries, unscaled).
  void ray(int index, double* ray);
  // Replaces LP `index`'s reported point (the triple solution() returns).
  void set_point(int index, const double* col_value, const double* col_dual,
                 const double* row_dual);
  void adjoint(const double* const* dl_dx, const double* const* dl_dy, const double* dl_df,
               double* const* dl_dc, double* const* dl_drl, double* const* dl_dru,
               double* const* dl_dl, double* const* dl_du, sankhya_gb300_adjoint_info* info);
  // Refines every converged, nondegenerate LP's reported point by its active-set solve;
  // items (load order) receive the new statuses, objectives and residuals.
  void polish(sankhya_gb300_batch_item* items, sankhya_gb300_adjoint_info* info);
  int count() const { return count_; }
  int distinct_matrices() const { return static_cast<int>(mats_.size()); }
  // The schedule of the next solves: lanes per row or column (1, 2, 4, 8, 16 or 32) and
  // threads per LP (128, 256 or 512); 0 and 0 let each solve pick it (autotune).
  void set_schedule(int lanes, int threads);
  // The schedule the last solve ran with, and the seconds its autotuning took (0 if the
  // schedule was set).
  void last_schedule(int* lanes, int* threads, double* tune_seconds) const;

 private:
  void require_loaded() const;
  // Times every candidate schedule on a sample of the batch (a few hundred steps of up to
  // four LPs per SM, spread over the size order) and returns the fastest.
  void autotune(BatchBuffers b, bool mixed, int* lanes, int* threads);
  void ensure_adjoint_buffers();
  AdjointBuffers adjoint_buffers();
  void finish_adjoint(double* const* dl_dc, double* const* dl_drl, double* const* dl_dru,
                      double* const* dl_dl, double* const* dl_du,
                      sankhya_gb300_adjoint_info* info);

  int device_ = 0;
  int sched_lanes_ = 0, sched_threads_ = 0;        // 0: autotune
  int last_lanes_ = 1, last_threads_ = kBatchThreads;
  double last_tune_seconds_ = 0.0;
  std::vector<int> order_;                         // the solve order (largest LP first)
  DeviceArray<int> d_tune_order_;
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
  // Mixed precision (allocated on the first mixed solve).
  bool mixed_ready_ = false;
  DeviceArray<float> csc_f_, csr_f_;
  DeviceArray<float> u0_, u1_, u_sum_, u_rst_, cf_, lf_, uf_, uc0_, uc1_, u_best_;
  DeviceArray<float2> ud_;
  DeviceArray<float> v0_, v1_, v_sum_, v_rst_, gu_, gl_, yhat_, vc0_, vc1_, v_best_;
  DeviceArray<long long> refinements_;
  BatchBuffers buffers_{};  // of the last solve
  // Adjoint (allocated on first use).
  bool adjoint_ready_ = false;
  DeviceArray<double> a_gx_, a_gy_, a_gf_, a_dc_, a_dl_, a_du_, a_drl_, a_dru_;
  DeviceArray<double> a_kw_[kAdjVectors];
  DeviceArray<int> a_bcol_, a_cpos_, a_rrow_, a_rpos_, a_kcp_, a_krp_, a_kci_, a_kri_;
  DeviceArray<double> a_kcv_, a_krv_;
  DeviceArray<long long> a_knz_;
  int a_smem_vec_ = 0;
  DeviceArray<signed char> a_cs_, a_rs_;
  DeviceArray<AdjointOutcome> a_out_;
  long long total_n_ = 0, total_m_ = 0, mat_n_ = 0, mat_m_ = 0;
};

}  // namespace sgb

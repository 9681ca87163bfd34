// engine.hpp -- host side of the GB300 PDHG engine (one LP, one device).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "chunks.cuh"
#include "kernels.cuh"
#include "mixed.cuh"
#include "sankhya_gb300.h"

namespace sgb {

// A named NVTX range for the lifetime of the object, marking an engine phase on a profiler's
// timeline (nsys, or ncu's --nvtx filters). The names follow SANKHYA's profiler scopes. With no
// tool attached NVTX calls return at once; without the NVTX headers this is empty.
struct Trace {
  explicit Trace(const char* name);
  ~Trace();
  Trace(const Trace&) = delete;
  Trace& operator=(const Trace&) = delete;
};

// Raised inside the engine and turned into a status code at the C boundary.
struct EngineError {
  int code;
  std::string message;
};

// Throws EngineError on any CUDA failure, with the call site in the message.
void cuda_check(cudaError_t err, const char* what, const char* file, int line);
#define SGB_CUDA(call) ::sgb::cuda_check((call), #call, __FILE__, __LINE__)

template <typename T>
struct DeviceArray {
  T* ptr = nullptr;
  size_t count = 0;
  DeviceArray() = default;
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  ~DeviceArray() { release(); }
  void allocate(size_t n);
  void upload(const T* host, size_t n, cudaStream_t s);
  // n entries followed by `pad` zeroed ones (count stays n).
  void allocate_padded(size_t n, size_t pad, cudaStream_t s);
  void upload_padded(const T* host, size_t n, size_t pad, cudaStream_t s);
  void release();
};

// Entries of the step-size factor table (decisions.cuh, step_factors): 16 MB of double2.
constexpr long long kStepFactorTable = 1LL << 20;

class Engine {
 public:
  explicit Engine(int device);
  ~Engine();

  void load(const sankhya_gb300_lp& lp);
  void solve(const sankhya_gb300_params& params, sankhya_gb300_result* result);
  void solution(double* col_value, double* col_dual, double* row_dual);
  void scaling(long long seed, double* row_scale, double* col_scale, double* scaled_values,
               double* spectral_norm);
  void spmv(int op, int scaled, const double* in, double* out);
  // The same product on caller-owned DEVICE buffers, enqueued on `stream` (nullptr: the
  // engine's stream) with the fixed scratch of noalloc_scratch(): allocates no memory.
  void spmv_noalloc(int op, int scaled, const double* in, double* out, cudaStream_t stream);
  void time_kernels(int reps, double* ms);

  int device() const { return device_; }

 private:
  void require_loaded() const;
  void precondition(long long seed);
  double power_iteration(long long seed);
  void init_iterates(const sankhya_gb300_params& p);
  void build_graphs(int steps);
  void build_mixed_graphs(int steps);
  void destroy_graphs();
  void fill_buffers();
  void fill_mixed_buffers();
  void allocate_mixed();
  // Runs CUDA graphs of `graph_steps_` steps until the control block behind `snapshot` says
  // done, the time limit passes or the interrupt flag is raised.
  void run_graphs(const sankhya_gb300_params& p, double t0, cudaGraphExec_t* graphs,
                  Ctl* snapshot, bool forward_log, long long iteration_offset, int* stop_status);
  void final_evaluation();
  // The tile products' error word (tickets_ slot 3, zero after load) and its check.
  unsigned int* product_error() const { return tickets_.ptr + 3; }
  void check_product_error();
  void setup(const sankhya_gb300_params& p, sankhya_gb300_result* r, double* norm);
  void solve_fp64(const sankhya_gb300_params& p, sankhya_gb300_result* r, double t0);
  void solve_mixed(const sankhya_gb300_params& p, sankhya_gb300_result* r, double t0);
  void report(const sankhya_gb300_params& p, const Ctl& c, bool converged, long long iterations,
              long long restarts, int stop_status, sankhya_gb300_result* r);

  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  int num_sms_ = 0;
  bool loaded_ = false;
  bool solved_ = false;
  bool scaled_ = false;

  // Problem dimensions and host-side scalars.
  int m_ = 0, n_ = 0;
  long long nnz_ = 0;
  double sense_ = 1.0, offset_ = 0.0;
  double bound_norm_ = 0.0, cost_norm_ = 0.0;
  int ntiles_csr_ = 0, ntiles_csc_ = 0;
  int nlong_csr_ = 0, nlong_csc_ = 0;
  int nchunks_csr_ = 0, nchunks_csc_ = 0;
  int lanes_csr_ = 1, lanes_csc_ = 1;
  int grid_csr_ = 1, grid_csc_ = 1;
  // The FP32 evaluation kernels' tile layout (same chunks of long rows, `lanes` threads per
  // row).
  int ntiles_csr_f_ = 0, ntiles_csc_f_ = 0;
  int lanes_csr_f_ = 1, lanes_csc_f_ = 1;
  int grid_csr_f_ = 1, grid_csc_f_ = 1;
  DeviceArray<Tile> csc_tiles_f_, csr_tiles_f_;
  // The FP64 step passes' gathered-vector windows per layout (CSC / CSR): tile -> window
  // id, the {lo, len} list, the capacity, and the grid and dynamic shared memory of the step
  // kernel that stages them.
  struct StepLayout {
    DeviceArray<int> tile_win;
    DeviceArray<int2> windows;
    int wmax = 0;
    int nwindows = 0;
    int grid = 1;
    int smem = 0;
    double staged = 0.0;  // share of the nonzeros gathered from a staged window
  };
  StepLayout step_csc_, step_csr_;
  // The FP32 step passes' chunk layouts (chunks.cuh): CSC (column pass) and CSR (row pass).
  // A split layout owns its main and outer index arrays (and the maps from their entries to
  // the full layout's, through which each solve fills their values); otherwise it reads the
  // full layout's arrays.
  struct ChunkDev {
    DeviceArray<Tile> chunks;
    DeviceArray<int2> orounds;
    DeviceArray<LongRow> longs;
    DeviceArray<ChunkSeg> segs;
    DeviceArray<int> seg_start, oround_start;
    DeviceArray<int> ptr, idx, map, optr, oidx, omap;
    DeviceArray<float> fval, foval, fouter;
    DeviceArray<double> pieces;  // piece partials (NP per piece)
    int nlong = 0, npieces = 0, wmax = 0, grid = 1, smem = 0, nrows = 0;
    bool split = false;
    long long nmain = 0, nouter = 0;
    double staged = 0.0;    // share of the nonzeros gathered from a staged window
    double coverage = 0.0;  // share the windows would hold over the whole layout
  };
  ChunkDev ck_csc_f_, ck_csr_f_;
  void plan_layout(ChunkDev& D, const std::vector<int>& ptr, const int* idx, int lines,
                   int extent, int pass, int window_cap);
  void fill_split_values();
  ChunkSet<float> chunk_set(const ChunkDev& D, const int* full_ptr, const int* full_idx,
                            const float* full_val) const;

  // Pattern (shared by scaled and unscaled values).
  DeviceArray<int> csc_ptr_, csc_idx_, csr_ptr_, csr_idx_;
  DeviceArray<Tile> csc_tiles_, csr_tiles_;
  DeviceArray<LongRow> csc_longs_, csr_longs_;
  // Values: unscaled (evaluation) and scaled (iterations), both layouts.
  DeviceArray<double> csc_raw_, csr_raw_, csc_s_, csr_s_;
  // Unscaled vectors.
  DeviceArray<double> cost_, col_cost_, l_, u_, rl_, ru_;
  // The step-size factors for iteration counts below kStepFactorTable (filled once).
  DeviceArray<double2> step_factors_;
  // Scaled vectors and scaling.
  DeviceArray<double> cs_, ls_, us_, rls_, rus_, dr_, dc_, row_acc_, col_acc_;
  // Iterates.
  DeviceArray<double> x0_, x1_, y0_, y1_, x_sum_, y_sum_, x_rst_, y_rst_;
  DeviceArray<double> xu0_, xu1_, yu0_, yu1_, reduced_, best_x_, best_y_;
  DeviceArray<double2> xd_;  // (2x' - x, x' - x) per column
  // Reductions.
  DeviceArray<double> part_primal_, part_dual_, part_rows0_, part_cols_, part_rows1_;
  DeviceArray<double> chunk_primal_, chunk_dual_, chunk_cols_, chunk_rows_, chunk_spmv_;
  DeviceArray<double> scalars_, power_v_, power_av_, power_norms_;
  DeviceArray<unsigned int> tickets_;  // setup-kernel last-block counters
  DeviceArray<Ctl> ctl_;

  Ctl* snapshot_ = nullptr;  // pinned host, two slots
  cudaGraphExec_t graph_exec_[2] = {nullptr, nullptr};
  int graph_steps_ = 0;
  cudaEvent_t done_event_[2] = {nullptr, nullptr};
  cudaEvent_t timing_[2] = {nullptr, nullptr};
  long long launches_ = 0;  // engine kernels launched by the current solve
  long long graphs_launched_ = 0;

  StepBuffers step_{};
  EvalBuffers eval_{};

  // Mixed method (allocated on its first solve).
  int last_precision_ = SANKHYA_GB300_FP64;
  bool mixed_ready_ = false;
  MixedBuffers mixed_{};
  DeviceArray<float> csc_f_, csr_f_;
  DeviceArray<float> u0f_, u1f_, v0f_, v1f_, usumf_, vsumf_, urstf_, vrstf_;
  DeviceArray<float> cf_, lf_, uf_, gu_, gl_, yhat_, uc0_, uc1_, vc0_, vc1_, ubest_, vbest_;
  DeviceArray<float> csf_;   // scaled cost in FP32
  DeviceArray<float> duf_;           // u' - u per column
  DeviceArray<float> auf0_, auf1_;   // A u per row, double-buffered with u
  DeviceArray<double> anchor_x_, anchor_y_, ax64_, aty64_;
  DeviceArray<Ctl> ctl_mixed_;
  Ctl* snapshot_mixed_ = nullptr;  // pinned host, two slots
  cudaGraphExec_t mgraph_exec_[2] = {nullptr, nullptr};
  int mgraph_steps_ = 0;
  double bound_norm_s_ = 0.0, cost_norm_s_ = 0.0;  // scaled problem norms
  long long extra_launches_ = 0;
};

size_t estimate_memory(long long rows, long long cols, long long nnz, int precision);

// The step passes' chunk layout of one matrix layout (layout.cu): `ptr` / `idx` its lines
// and indices over a gathered vector of `extent` elements, `cap` entries per chunk, `wmax`
// the window capacity, `grid` blocks, `elem_bytes` the gathered element's size. Windows are
// kept over every entry when they hold at least `full_min` of them; between `split_min` and
// that, the layout is split into main and outer parts; below it, nothing is staged. A split
// layout's outer entries are summed in rounds of at most `outer_round_cap` entries.
struct ChunkPlan {
  int cap = 0, grid = 1, wmax = 0, npieces = 0;
  bool split = false, error = false;
  double coverage = 0.0, staged = 0.0;
  std::vector<Tile> chunks;
  std::vector<int2> orounds;
  std::vector<LongRow> longs;
  std::vector<ChunkSeg> segs;
  std::vector<int> seg_start, oround_start;
  std::vector<int> ptr, idx, map, optr, oidx, omap;  // split layouts only
};
ChunkPlan plan_chunks(const std::vector<int>& ptr, const int* idx, int lines, int extent, int cap,
                      int wmax, int grid, int elem_bytes, double split_min, double full_min,
                      int outer_round_cap);

// The status a tile product's error word maps to: 0 = ok, otherwise a device error.
int product_error_status(unsigned int word);

// Throws EngineError (ARGUMENT / MODEL) when an LP is malformed.
void validate_lp(const sankhya_gb300_lp& lp);

// Row tiles of a CSR / CSC pattern (see tiles.cuh).
void build_tiles(const std::vector<int>& ptr, int lines, int lanes, int threads,
                 std::vector<Tile>* tiles, std::vector<LongRow>* longs, int* nchunks);

// Gathered-vector windows of one tile layout (see tiles.cuh): `idx` is the layout's index
// array over a gathered vector of `extent` elements, `wmax` the window capacity.
// Returns the number of nonzeros whose index falls in their tile's window.
long long build_windows(const std::vector<Tile>& tiles, const int* idx, int extent, int wmax,
                        std::vector<int>* tile_win, std::vector<int2>* windows);

}  // namespace sgb

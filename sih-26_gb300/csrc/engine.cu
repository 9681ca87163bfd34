// engine.cu -- host driver of the GB300 PDHG engine.
//
// Follows src/pdhg/pdhg.cpp:76-568 step for step, with every vector on the device:
//   setup     device Ruiz x10 + Pock-Chambolle (src/la/scaling.cpp:111-159) on both the CSC
//             and the CSR copy, power iteration (src/la/scaling.cpp:161-194) from the same
//             std::mt19937 start, x0 = proj(0), y0 = 0 (src/pdhg/pdhg.cpp:140-147);
//   loop      CUDA graphs of `steps_per_poll` attempted steps, each step = k_primal + k_dual,
//             with the evaluation kernels after every kEvalStride steps (a step that falls
//             due for an evaluation holds the steps after it until the evaluation has run);
//             the host launches graph k+1 before it reads the status snapshot graph k
//             copied out, so the device never waits on the host;
//   report    one final evaluation of (best_x, best_y) on the device
//             (src/pdhg/pdhg.cpp:487-567), status and message assembled here.
// The reference checks the clock at every step; this engine checks it, and the
// SolveControl interrupt flag, at every snapshot (every `steps_per_poll` steps).
#include "engine.hpp"

#include "batch.cuh"
#include "qp.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstddef>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <limits>
#include <random>
#include <thread>

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define SGB_HAVE_NVTX 1
#endif
#endif

namespace sgb {

#ifdef SGB_HAVE_NVTX
Trace::Trace(const char* name) { nvtxRangePushA(name); }
Trace::~Trace() { nvtxRangePop(); }
#else
Trace::Trace(const char*) {}
Trace::~Trace() {}
#endif

void cuda_check(cudaError_t err, const char* what, const char* file, int line) {
  if (err == cudaSuccess) return;
  char buf[512];
  std::snprintf(buf, sizeof(buf), "CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(err),
                cudaGetErrorString(err), what, file, line);
  const int code = (err == cudaErrorMemoryAllocation) ? SANKHYA_GB300_ERROR_MEMORY
                                                      : SANKHYA_GB300_ERROR_DEVICE;
  throw EngineError{code, buf};
}

template <typename T>
void DeviceArray<T>::allocate(size_t n) {
  release();
  count = n;
  if (n > 0) SGB_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
}
template <typename T>
void DeviceArray<T>::upload(const T* host, size_t n, cudaStream_t s) {
  allocate(n);
  if (n > 0) SGB_CUDA(cudaMemcpyAsync(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
}
template <typename T>
void DeviceArray<T>::allocate_padded(size_t n, size_t pad, cudaStream_t s) {
  allocate(n + pad);
  if (n + pad > 0) SGB_CUDA(cudaMemsetAsync(ptr, 0, (n + pad) * sizeof(T), s));
  count = n;
}
template <typename T>
void DeviceArray<T>::upload_padded(const T* host, size_t n, size_t pad, cudaStream_t s) {
  allocate_padded(n, pad, s);
  if (n > 0) SGB_CUDA(cudaMemcpyAsync(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
}
template <typename T>
void DeviceArray<T>::release() {
  if (ptr != nullptr) cudaFree(ptr);
  ptr = nullptr;
  count = 0;
}
template struct DeviceArray<int>;
template struct DeviceArray<int2>;
template struct DeviceArray<double2>;
template struct DeviceArray<float2>;
template struct DeviceArray<Tile>;
template struct DeviceArray<LongRow>;
template struct DeviceArray<unsigned int>;
template struct DeviceArray<double>;
template struct DeviceArray<float>;
template struct DeviceArray<Ctl>;
template struct DeviceArray<BatchMatrix>;
template struct DeviceArray<BatchInstance>;
template struct DeviceArray<BatchOutcome>;
template struct DeviceArray<AdjointOutcome>;
template struct DeviceArray<signed char>;
template struct DeviceArray<long long>;
template struct DeviceArray<ChunkSeg>;
template struct DeviceArray<QpChunk>;
template struct DeviceArray<QpCtl>;
template struct DeviceArray<QpHist>;

namespace {

double now_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

bool finite_bound_host(double v) { return !(std::isinf(v) || std::fabs(v) >= 1e30); }

}  // namespace

// Greedy row tiles: consecutive rows while the tile has at most min(kMaxTileRows,
// threads / lanes) rows and at most kCap nonzeros; a row longer than kCap becomes chunk tiles
// of kCap entries each, listed as a LongRow so its chunk partials can be combined in chunk
// order. With one lane per row, a row of more than kWarpRowMin entries (and at most kCap)
// gets a tile of its own, which one warp sums (see run_tiles).
void build_tiles(const std::vector<int>& ptr, int lines, int lanes, int threads,
                 std::vector<Tile>* tiles, std::vector<LongRow>* longs, int* nchunks) {
  tiles->clear();
  longs->clear();
  *nchunks = 0;
  const int max_rows = std::min(kMaxTileRows, threads / lanes);
  int r = 0;
  while (r < lines) {
    const int len = ptr[r + 1] - ptr[r];
    if (len > kCap) {
      LongRow lr{r, *nchunks, 0};
      for (int k = ptr[r]; k < ptr[r + 1]; k += kCap) {
        const int k1 = std::min(k + kCap, ptr[r + 1]);
        tiles->push_back(Tile{r, -(*nchunks) - 1, k, k1});
        ++*nchunks;
        ++lr.nchunks;
      }
      longs->push_back(lr);
      ++r;
      continue;
    }
    const int begin = r;
    ++r;
    const bool warp_row = lanes == 1 && len > kWarpRowMin;
    while (!warp_row && r < lines && r - begin < max_rows && ptr[r + 1] - ptr[r] <= kCap &&
           (lanes != 1 || ptr[r + 1] - ptr[r] <= kWarpRowMin) &&
           ptr[r + 1] - ptr[begin] <= kCap) {
      ++r;
    }
    tiles->push_back(Tile{begin, r, ptr[begin], ptr[r]});
  }
}

// Windows: first every tile's own best range -- the start lo for which [lo, lo + wmax) holds
// the most of the tile's entries, centred among the starts that do and rounded down to a
// multiple of 4 -- computed on all host threads (tiles are independent). Then, in tile
// order, a tile joins the current window when its own best start lies within wmax / 16 of
// the window's; otherwise it opens a new window at its own best start. A tile with fewer
// than 1/8 of its entries in its best range gathers from global memory. A window whose tiles
// would gather fewer than wmax / 32 entries from it is dropped: staging costs one bulk copy
// of the whole window, about a thirty-second of a random gather per element.
long long build_windows(const std::vector<Tile>& tiles, const int* idx, int extent, int wmax,
                        std::vector<int>* tile_win, std::vector<int2>* windows) {
  const int ntiles = static_cast<int>(tiles.size());
  tile_win->assign(static_cast<size_t>(ntiles), -1);
  windows->clear();
  if (wmax <= 0 || ntiles == 0 || extent <= 0) return 0;
  const int ext4 = (extent + 3) & ~3;
  if (ext4 <= wmax) {  // the whole vector fits: one window for every tile
    windows->push_back(make_int2(0, ext4));
    tile_win->assign(static_cast<size_t>(ntiles), 0);
    long long all = 0;
    for (const Tile& t : tiles) all += t.k1 - t.k0;
    return all;
  }
  std::vector<int> best_lo(static_cast<size_t>(ntiles)), best_count(static_cast<size_t>(ntiles));
  const auto scan = [&](int t0, int t1) {
    std::vector<int> v;
    for (int t = t0; t < t1; ++t) {
      const Tile& tile = tiles[static_cast<size_t>(t)];
      v.assign(idx + tile.k0, idx + tile.k1);
      std::sort(v.begin(), v.end());
      int best = 0, bl = 0, br = 0;
      for (int r = 0, l = 0; r < static_cast<int>(v.size()); ++r) {
        while (v[r] - v[l] >= wmax) ++l;
        if (r - l + 1 > best) {
          best = r - l + 1;
          bl = l;
          br = r;
        }
      }
      long long lo = 0;
      if (best > 0) {
        const long long lo_min = static_cast<long long>(v[br]) - wmax + 1, lo_max = v[bl];
        lo = lo_min + (lo_max - lo_min) / 2;
      }
      lo = std::max(0LL, std::min(lo, static_cast<long long>(ext4 - wmax)));
      best_lo[static_cast<size_t>(t)] = static_cast<int>(lo) & ~3;
      best_count[static_cast<size_t>(t)] = best;
    }
  };
  const int workers = std::max(1, std::min<int>(16, static_cast<int>(std::thread::hardware_concurrency())));
  if (workers == 1 || ntiles < 64) {
    scan(0, ntiles);
  } else {
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; ++w) {
      const int t0 = static_cast<int>(static_cast<long long>(ntiles) * w / workers);
      const int t1 = static_cast<int>(static_cast<long long>(ntiles) * (w + 1) / workers);
      pool.emplace_back(scan, t0, t1);
    }
    for (auto& th : pool) th.join();
  }
  std::vector<long long> used;  // entries each window serves (its tiles' best counts)
  int current = -1;
  for (int t = 0; t < ntiles; ++t) {
    const Tile& tile = tiles[static_cast<size_t>(t)];
    const int entries = tile.k1 - tile.k0;
    const int best = best_count[static_cast<size_t>(t)];
    if (entries == 0 || best * 8 < entries) continue;
    const int lo = best_lo[static_cast<size_t>(t)];
    if (current < 0 || std::abs(lo - (*windows)[static_cast<size_t>(current)].x) > wmax / 16) {
      windows->push_back(make_int2(lo, wmax));
      used.push_back(0);
      current = static_cast<int>(windows->size()) - 1;
    }
    (*tile_win)[static_cast<size_t>(t)] = current;
    used[static_cast<size_t>(current)] += best;
  }
  // Drop windows that do not pay for their staging, renumbering the rest.
  std::vector<int> remap(windows->size(), -1);
  std::vector<int2> kept;
  for (size_t w = 0; w < windows->size(); ++w) {
    if (used[w] * 32 >= wmax) {
      remap[w] = static_cast<int>(kept.size());
      kept.push_back((*windows)[w]);
    }
  }
  for (int& w : *tile_win) {
    if (w >= 0) w = remap[static_cast<size_t>(w)];
  }
  windows->swap(kept);
  long long covered = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int w = (*tile_win)[static_cast<size_t>(t)];
    if (w < 0) continue;
    const int2 r = (*windows)[static_cast<size_t>(w)];
    for (int k = tiles[static_cast<size_t>(t)].k0; k < tiles[static_cast<size_t>(t)].k1; ++k) {
      covered += static_cast<unsigned>(idx[k] - r.x) < static_cast<unsigned>(r.y);
    }
  }
  return covered;
}

namespace {

std::string format(const char* fmt, ...) __attribute__((format(printf, 1, 2)));
std::string format(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return buf;
}

}  // namespace

size_t estimate_memory(long long rows, long long cols, long long nnz, int precision) {
  const size_t m = static_cast<size_t>(rows < 0 ? 0 : rows);
  const size_t n = static_cast<size_t>(cols < 0 ? 0 : cols);
  const size_t z = static_cast<size_t>(nnz < 0 ? 0 : nnz);
  size_t bytes = 0;
  bytes += (m + 1 + n + 1) * sizeof(int) + 2 * z * sizeof(int);  // CSR + CSC pattern
  bytes += (m + n) * sizeof(int2);                                // tiles (upper bound)
  bytes += 4 * z * sizeof(double);      // unscaled + scaled values, both layouts
  bytes += 18 * n * sizeof(double);     // column vectors (see Engine members)
  bytes += 14 * m * sizeof(double);     // row vectors
  if (precision == SANKHYA_GB300_MIXED) {
    bytes += 2 * z * sizeof(float) + (10 * n + 8 * m) * sizeof(float);
  }
  // Fixed: the kernels' device code (a 5.8 MB fatbin, loaded at the first launch, after a
  // caller's memory check), the partial-sum buffers and the control block; and the 16 MB
  // table of step-size factors.
  bytes += 16u << 20;
  bytes += static_cast<size_t>(kStepFactorTable) * sizeof(double2);
  return bytes;
}

Engine::Engine(int device) : device_(device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "no CUDA device is available"};
  }
  if (device < 0 || device >= count) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT,
                      format("device %d does not exist (%d present)", device, count)};
  }
  SGB_CUDA(cudaSetDevice(device));
  SGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SGB_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device));
  SGB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&snapshot_), 2 * sizeof(Ctl),
                         cudaHostAllocDefault));
  SGB_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&snapshot_mixed_), 2 * sizeof(Ctl),
                         cudaHostAllocDefault));
  for (auto& ev : done_event_) SGB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  for (auto& ev : timing_) SGB_CUDA(cudaEventCreate(&ev));
  ctl_.allocate(1);
  SGB_CUDA(cudaMemset(ctl_.ptr, 0, sizeof(Ctl)));
  ctl_mixed_.allocate(1);
  SGB_CUDA(cudaMemset(ctl_mixed_.ptr, 0, sizeof(Ctl)));
  if (!configure_tile_kernels() || !configure_mixed_kernels()) {
    throw EngineError{SANKHYA_GB300_ERROR_DEVICE,
                      format("device %d refused the kernels' shared-memory limits", device)};
  }
}

Engine::~Engine() {
  cudaSetDevice(device_);
  destroy_graphs();
  for (auto& ev : done_event_) {
    if (ev != nullptr) cudaEventDestroy(ev);
  }
  for (auto& ev : timing_) {
    if (ev != nullptr) cudaEventDestroy(ev);
  }
  if (snapshot_ != nullptr) cudaFreeHost(snapshot_);
  if (snapshot_mixed_ != nullptr) cudaFreeHost(snapshot_mixed_);
  if (stream_ != nullptr) cudaStreamDestroy(stream_);
}

void Engine::destroy_graphs() {
  for (auto& g : graph_exec_) {
    if (g != nullptr) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  for (auto& g : mgraph_exec_) {
    if (g != nullptr) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  graph_steps_ = 0;
  mgraph_steps_ = 0;
}

// The FP32 copies, the correction problem and the FP64 anchor of the mixed method.
void Engine::allocate_mixed() {
  if (mixed_ready_) return;
  cudaStream_t s = stream_;
  const size_t z = static_cast<size_t>(nnz_), n = static_cast<size_t>(n_);
  const size_t m = static_cast<size_t>(m_);
  csc_f_.allocate_padded(z, kPad, s);
  csr_f_.allocate_padded(z, kPad, s);
  // kPad elements of padding, as for the FP64 vectors (staged slices and windows).
  for (DeviceArray<float>* a : {&u0f_, &u1f_, &usumf_, &urstf_, &cf_, &lf_, &uf_, &uc0_, &uc1_,
                                &ubest_, &csf_, &duf_}) {
    a->allocate(n + kPad);
  }
  for (DeviceArray<float>* a : {&v0f_, &v1f_, &vsumf_, &vrstf_, &gu_, &gl_, &yhat_, &vc0_, &vc1_,
                                &vbest_, &auf0_, &auf1_}) {
    a->allocate(m + kPad);
  }
  for (DeviceArray<double>* a : {&anchor_x_, &aty64_}) a->allocate(n);
  for (DeviceArray<double>* a : {&anchor_y_, &ax64_}) a->allocate(m);
  for (ChunkDev* D : {&ck_csc_f_, &ck_csr_f_}) {
    if (!D->split) continue;
    D->fval.allocate_padded(static_cast<size_t>(D->nmain), kPad, s);
    D->foval.allocate_padded(static_cast<size_t>(D->nouter), kPad, s);
    D->fouter.allocate_padded(static_cast<size_t>(D->nrows), kPad, s);
  }
  fill_mixed_buffers();
  mixed_ready_ = true;
}

void Engine::fill_mixed_buffers() {
  MixedBuffers& b = mixed_;
  b.ctl = ctl_mixed_.ptr;
  b.csc = TileSet<float>{csc_ptr_.ptr,   csc_idx_.ptr,  csc_f_.ptr,   csc_tiles_f_.ptr,
                         csc_longs_.ptr, ntiles_csc_f_, nlong_csc_,   nchunks_csc_,
                         n_,             lanes_csc_f_};
  b.csr = TileSet<float>{csr_ptr_.ptr,   csr_idx_.ptr,  csr_f_.ptr,   csr_tiles_f_.ptr,
                         csr_longs_.ptr, ntiles_csr_f_, nlong_csr_,   nchunks_csr_,
                         m_,             lanes_csr_f_};
  b.u[0] = u0f_.ptr;
  b.u[1] = u1f_.ptr;
  b.v[0] = v0f_.ptr;
  b.v[1] = v1f_.ptr;
  b.u_sum = usumf_.ptr;
  b.v_sum = vsumf_.ptr;
  b.u_rst = urstf_.ptr;
  b.v_rst = vrstf_.ptr;
  b.du = duf_.ptr;
  b.au[0] = auf0_.ptr;
  b.au[1] = auf1_.ptr;
  b.cf = cf_.ptr;
  b.lf = lf_.ptr;
  b.uf = uf_.ptr;
  b.cs = csf_.ptr;
  b.gu = gu_.ptr;
  b.gl = gl_.ptr;
  b.yhat = yhat_.ptr;
  b.uc[0] = uc0_.ptr;
  b.uc[1] = uc1_.ptr;
  b.vc[0] = vc0_.ptr;
  b.vc[1] = vc1_.ptr;
  b.u_best = ubest_.ptr;
  b.v_best = vbest_.ptr;
  b.step_factors = step_factors_.ptr;
  b.step_factors_n = kStepFactorTable;
  b.part_primal = part_primal_.ptr;
  b.part_dual = part_dual_.ptr;
  b.csc_k = chunk_set(ck_csc_f_, csc_ptr_.ptr, csc_idx_.ptr, csc_f_.ptr);
  b.csr_k = chunk_set(ck_csr_f_, csr_ptr_.ptr, csr_idx_.ptr, csr_f_.ptr);
  b.piece_primal = ck_csc_f_.pieces.ptr;
  b.piece_dual = ck_csr_f_.pieces.ptr;
  b.part_rows0 = part_rows0_.ptr;
  b.part_cols = part_cols_.ptr;
  b.part_rows1 = part_rows1_.ptr;
  b.chunk_cols = chunk_cols_.ptr;
  b.chunk_rows = chunk_rows_.ptr;
  b.grid_primal = grid_csc_f_;
  b.grid_dual = grid_csr_f_;
  b.grid_step_primal = ck_csc_f_.grid;
  b.grid_step_dual = ck_csr_f_.grid;
  b.smem_primal = ck_csc_f_.smem;
  b.smem_dual = ck_csr_f_.smem;
  b.m = m_;
  b.n = n_;
}

void Engine::build_mixed_graphs(int steps) {
  if (mgraph_steps_ == steps && mgraph_exec_[0] != nullptr) return;
  for (auto& g : mgraph_exec_) {
    if (g != nullptr) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  for (int slot = 0; slot < 2; ++slot) {
    cudaGraph_t graph = nullptr;
    SGB_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; ++k) {
      launch_mixed_step(mixed_, stream_);
      if ((k + 1) % kEvalStride == 0 || k + 1 == steps) launch_mixed_evaluation(mixed_, stream_);
    }
    cudaMemcpyAsync(snapshot_mixed_ + slot, ctl_mixed_.ptr, sizeof(Ctl), cudaMemcpyDeviceToHost,
                    stream_);
    const cudaError_t end = cudaStreamEndCapture(stream_, &graph);
    SGB_CUDA(end);
    const cudaError_t inst = cudaGraphInstantiate(&mgraph_exec_[slot], graph, 0);
    cudaGraphDestroy(graph);
    SGB_CUDA(inst);
  }
  mgraph_steps_ = steps;
}

void Engine::require_loaded() const {
  if (!loaded_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no LP has been loaded"};
}

// Model::validate's structural and numeric checks (src/core/model.cpp:175-183 and the bound
// checks) on an LP handed across the boundary.
void validate_lp(const sankhya_gb300_lp& lp) {
  if (lp.rows < 0 || lp.cols < 0 || lp.col_starts == nullptr) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "bad LP dimensions or null column starts"};
  }
  const int m = lp.rows, n = lp.cols;
  const long long nnz = lp.col_starts[n];
  if (lp.col_starts[0] != 0 || nnz < 0) {
    throw EngineError{SANKHYA_GB300_ERROR_MODEL, "column starts must begin at 0"};
  }
  for (int j = 0; j < n; ++j) {
    if (lp.col_starts[j + 1] < lp.col_starts[j]) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL, "column starts are not monotone"};
    }
  }
  for (long long k = 0; k < nnz; ++k) {
    const int i = lp.row_index[k];
    if (i < 0 || i >= m) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL, format("row index %d out of range", i)};
    }
    if (!std::isfinite(lp.values[k])) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL,
                        format("matrix entry %lld is %g, which is not a usable coefficient", k,
                               lp.values[k])};
    }
  }
  for (int j = 0; j < n; ++j) {
    if (!std::isfinite(lp.col_cost[j]) || std::isnan(lp.col_lower[j]) ||
        std::isnan(lp.col_upper[j]) || lp.col_lower[j] > lp.col_upper[j]) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL, format("column %d has a bad cost or bound", j)};
    }
    for (int k = lp.col_starts[j] + 1; k < lp.col_starts[j + 1]; ++k) {
      if (lp.row_index[k] <= lp.row_index[k - 1]) {
        throw EngineError{SANKHYA_GB300_ERROR_MODEL,
                          format("column %d: row indices are not strictly ascending", j)};
      }
    }
  }
  for (int i = 0; i < m; ++i) {
    if (std::isnan(lp.row_lower[i]) || std::isnan(lp.row_upper[i]) ||
        lp.row_lower[i] > lp.row_upper[i]) {
      throw EngineError{SANKHYA_GB300_ERROR_MODEL, format("row %d has a bad bound", i)};
    }
  }
  if (std::isnan(lp.objective_offset)) {
    throw EngineError{SANKHYA_GB300_ERROR_MODEL, "objective offset is NaN"};
  }
  if (nnz > std::numeric_limits<int>::max()) {
    throw EngineError{SANKHYA_GB300_ERROR_MODEL, "more nonzeros than int32 indices address"};
  }
}

void Engine::load(const sankhya_gb300_lp& lp) {
  Trace trace("pdhg load");
  validate_lp(lp);
  const int m = lp.rows, n = lp.cols;
  const long long nnz = lp.col_starts[n];
  SGB_CUDA(cudaSetDevice(device_));
  destroy_graphs();
  loaded_ = solved_ = scaled_ = mixed_ready_ = false;
  m_ = m;
  n_ = n;
  nnz_ = nnz;
  sense_ = lp.sense < 0.0 ? -1.0 : 1.0;
  offset_ = lp.objective_offset;

  // CSC as given; CSR by a counting-sort transpose walking columns in ascending order, so
  // the column indices come out ascending inside each row (src/la/sparse.cpp:271-302).
  std::vector<int> cptr(lp.col_starts, lp.col_starts + n + 1);
  std::vector<int> rptr(static_cast<size_t>(m) + 1, 0);
  for (long long k = 0; k < nnz; ++k) ++rptr[static_cast<size_t>(lp.row_index[k]) + 1];
  for (int i = 0; i < m; ++i) rptr[i + 1] += rptr[i];
  std::vector<int> next(rptr.begin(), rptr.end() - 1);
  std::vector<int> ridx(static_cast<size_t>(nnz));
  std::vector<double> rval(static_cast<size_t>(nnz));
  for (int j = 0; j < n; ++j) {
    for (int k = cptr[j]; k < cptr[j + 1]; ++k) {
      const int slot = next[lp.row_index[k]]++;
      ridx[slot] = j;
      rval[slot] = lp.values[k];
    }
  }
  // Two tile layouts per pattern. FP64 kernels run one row per thread: GB300's FP64 pipe
  // charges per warp instruction, so lanes that sit out an epilogue or add up a row that is
  // split across lanes cost as much as working ones. The FP32 kernels are bound by memory
  // latency instead and split rows over `lanes` threads so every thread issues gathers.
  // The chunking of long rows does not depend on the lanes, so both layouts share it.
  std::vector<Tile> ctiles, rtiles, ctiles_f, rtiles_f;
  std::vector<LongRow> clongs, rlongs;
  int unused_chunks = 0;
  lanes_csc_ = 1;
  lanes_csr_ = 1;
  lanes_csc_f_ = wide_lanes(n > 0 ? static_cast<double>(nnz) / n : 1.0, kWideThreads);
  lanes_csr_f_ = wide_lanes(m > 0 ? static_cast<double>(nnz) / m : 1.0, kWideThreads);
  build_tiles(cptr, n, lanes_csc_, kTileThreads, &ctiles, &clongs, &nchunks_csc_);
  build_tiles(rptr, m, lanes_csr_, kTileThreads, &rtiles, &rlongs, &nchunks_csr_);
  {
    std::vector<LongRow> same;
    build_tiles(cptr, n, lanes_csc_f_, kWideThreads, &ctiles_f, &same, &unused_chunks);
    build_tiles(rptr, m, lanes_csr_f_, kWideThreads, &rtiles_f, &same, &unused_chunks);
  }
  ntiles_csc_ = static_cast<int>(ctiles.size());
  ntiles_csr_ = static_cast<int>(rtiles.size());
  ntiles_csc_f_ = static_cast<int>(ctiles_f.size());
  ntiles_csr_f_ = static_cast<int>(rtiles_f.size());
  nlong_csc_ = static_cast<int>(clongs.size());
  nlong_csr_ = static_cast<int>(rlongs.size());
  const int resident = tile_blocks_per_sm() * num_sms_;
  grid_csc_ = std::max(1, std::min(ntiles_csc_, resident));
  grid_csr_ = std::max(1, std::min(ntiles_csr_, resident));
  const int resident_f = mixed_blocks_per_sm() * num_sms_;
  grid_csc_f_ = std::max(1, std::min(ntiles_csc_f_, resident_f));
  grid_csr_f_ = std::max(1, std::min(ntiles_csr_f_, resident_f));
  int grid_c = std::max(grid_csc_, grid_csc_f_), grid_r = std::max(grid_csr_, grid_csr_f_);

  // Minimise-space cost and the norms of src/pdhg/pdhg.cpp:95-111, summed in the
  // reference's order on the host (they are computed once).
  std::vector<double> cost(static_cast<size_t>(n));
  double cost_sq = 0.0;
  for (int j = 0; j < n; ++j) {
    cost[j] = sense_ * lp.col_cost[j];
    cost_sq += cost[j] * cost[j];
  }
  cost_norm_ = std::sqrt(cost_sq);
  double bound_sq = 0.0;
  for (int i = 0; i < m; ++i) {
    const double b = finite_bound_host(lp.row_lower[i])
                         ? lp.row_lower[i]
                         : (finite_bound_host(lp.row_upper[i]) ? lp.row_upper[i] : 0.0);
    bound_sq += b * b;
  }
  bound_norm_ = std::sqrt(bound_sq);

  cudaStream_t s = stream_;
  const size_t z = static_cast<size_t>(nnz);

  // The step passes' windows of the gathered vector: the column passes gather y (m rows),
  // the row passes the packed (2x' - x, x' - x) (FP64) or du (FP32) (n columns).
  // SANKHYA_GB300_WINDOW_CAP caps the capacity (0 turns staging off), so tests can force
  // partial windows on small LPs; in the FP32 chunk layouts it also splits every layout whose
  // windows hold any entry, so tests run the split form.
  int cap = -1;
  if (const char* env = std::getenv("SANKHYA_GB300_WINDOW_CAP")) cap = std::max(0, std::atoi(env)) & ~3;
  const auto make_layout = [&](StepLayout& L, const std::vector<Tile>& tiles, const int* idx,
                               int extent, int pass) {
    int wmax = fp64_window_capacity(pass);
    if (cap >= 0) wmax = std::min(wmax, cap);
    std::vector<int> tile_win;
    std::vector<int2> windows;
    long long covered = build_windows(tiles, idx, extent, wmax, &tile_win, &windows);
    // A window leaves room for one block per SM, whose few warps cannot hide the latency of
    // the gathers that miss it; below kMinStagedShare the unstaged form (several blocks per
    // SM, every gather from L2) is faster, so the layout keeps no window. A fixed rule, not a
    // timing: the grid decides the order of the block partial sums, so it must not vary from
    // run to run.
    // (A capacity set through SANKHYA_GB300_WINDOW_CAP keeps its windows whatever their
    // share, so tests can run the partly staged form.)
    constexpr double kMinStagedShare = 0.95;
    if (cap < 0 && nnz > 0 &&
        static_cast<double>(covered) < kMinStagedShare * static_cast<double>(nnz)) {
      tile_win.assign(tile_win.size(), -1);
      windows.clear();
      covered = 0;
    }
    L.staged = nnz > 0 ? static_cast<double>(covered) / static_cast<double>(nnz) : 0.0;
    L.nwindows = static_cast<int>(windows.size());
    L.wmax = 0;
    for (const int2& w : windows) L.wmax = std::max(L.wmax, w.y);
    L.smem = fp64_step_smem(pass, L.wmax);
    const int per_sm = fp64_step_blocks_per_sm(pass, L.smem);
    L.grid = std::max(1, std::min(static_cast<int>(tiles.size()), per_sm * num_sms_));
    L.tile_win.upload(tile_win.data(), tile_win.size(), s);
    L.windows.upload(windows.data(), windows.size(), s);
  };
  make_layout(step_csc_, ctiles, lp.row_index, m, 0);
  make_layout(step_csr_, rtiles, ridx.data(), n, 1);
  plan_layout(ck_csc_f_, cptr, lp.row_index, n, m, 0, cap);
  plan_layout(ck_csr_f_, rptr, ridx.data(), m, n, 1, cap);
  grid_c = std::max({grid_c, step_csc_.grid, ck_csc_f_.grid});
  grid_r = std::max({grid_r, step_csr_.grid, ck_csr_f_.grid});

  // Row pointers are staged per tile in 16-byte units too: kPad entries of padding.
  csc_ptr_.upload_padded(cptr.data(), cptr.size(), kPad, s);
  csr_ptr_.upload_padded(rptr.data(), rptr.size(), kPad, s);
  // Index and value arrays carry kPad zero entries: a tile copy widened to 16-byte
  // boundaries may read up to 3 entries past the last nonzero.
  csc_idx_.upload_padded(lp.row_index, z, kPad, s);
  csc_raw_.upload_padded(lp.values, z, kPad, s);
  csr_idx_.upload_padded(ridx.data(), z, kPad, s);
  csr_raw_.upload_padded(rval.data(), z, kPad, s);
  csc_s_.allocate_padded(z, kPad, s);
  csr_s_.allocate_padded(z, kPad, s);
  csc_tiles_.upload(ctiles.data(), ctiles.size(), s);
  csr_tiles_.upload(rtiles.data(), rtiles.size(), s);
  csc_tiles_f_.upload(ctiles_f.data(), ctiles_f.size(), s);
  csr_tiles_f_.upload(rtiles_f.data(), rtiles_f.size(), s);
  csc_longs_.upload(clongs.data(), clongs.size(), s);
  csr_longs_.upload(rlongs.data(), rlongs.size(), s);
  cost_.upload(cost.data(), cost.size(), s);
  col_cost_.upload(lp.col_cost, static_cast<size_t>(n), s);
  l_.upload(lp.col_lower, static_cast<size_t>(n), s);
  u_.upload(lp.col_upper, static_cast<size_t>(n), s);
  rl_.upload(lp.row_lower, static_cast<size_t>(m), s);
  ru_.upload(lp.row_upper, static_cast<size_t>(m), s);
  // Every per-row and per-column vector carries kPad elements of padding: the step passes
  // stage a tile's operand slices widened to 4-element bounds, and their windows of the
  // gathered vector may end up to 3 elements past the last one.
  for (DeviceArray<double>* a : {&cs_, &ls_, &us_, &dc_, &col_acc_, &x0_, &x1_, &x_sum_, &x_rst_,
                                 &xu0_, &xu1_, &reduced_, &best_x_, &power_v_}) {
    a->allocate(static_cast<size_t>(n) + kPad);
  }
  xd_.allocate(static_cast<size_t>(n) + kPad);
  for (DeviceArray<double>* a : {&rls_, &rus_, &dr_, &row_acc_, &y0_, &y1_, &y_sum_, &y_rst_,
                                 &yu0_, &yu1_, &best_y_, &power_av_}) {
    a->allocate(static_cast<size_t>(m) + kPad);
  }
  const int pgrid = std::max(grid_c, grid_r) + num_sms_ * 8;
  part_primal_.allocate(static_cast<size_t>(grid_c));
  part_dual_.allocate(static_cast<size_t>(grid_r) * 2);
  part_rows0_.allocate(static_cast<size_t>(grid_r) * kEvalRowSlots);
  part_cols_.allocate(static_cast<size_t>(grid_c + 1) * kEvalColSlots);
  part_rows1_.allocate(static_cast<size_t>(grid_r) * kEvalRowSlots);
  chunk_primal_.allocate(static_cast<size_t>(nchunks_csc_) + 1);
  chunk_dual_.allocate(2 * static_cast<size_t>(nchunks_csr_) + 2);
  chunk_cols_.allocate(2 * static_cast<size_t>(nchunks_csc_) + 2);
  chunk_rows_.allocate(2 * static_cast<size_t>(nchunks_csr_) + 2);
  chunk_spmv_.allocate(static_cast<size_t>(std::max(nchunks_csc_, nchunks_csr_)) + 1);
  scalars_.allocate(static_cast<size_t>(pgrid) * 2 + 16);
  power_norms_.allocate(64);
  if (step_factors_.ptr == nullptr) {
    step_factors_.allocate(static_cast<size_t>(kStepFactorTable));
    launch_step_factors(step_factors_.ptr, kStepFactorTable, s);
  }
  tickets_.allocate(4);
  SGB_CUDA(cudaMemsetAsync(tickets_.ptr, 0, 4 * sizeof(unsigned int), s));
  SGB_CUDA(cudaStreamSynchronize(s));
  fill_buffers();
  loaded_ = true;
}

// One FP32 step pass's chunk layout: planned on the host (plan_chunks), uploaded, and its
// piece and split buffers allocated. Windows are kept over every entry when they hold at least
// 99.9% of them and the layout is split from 50% up; a capacity set through
// SANKHYA_GB300_WINDOW_CAP (window_cap >= 0) splits any layout whose windows hold an entry.
void Engine::plan_layout(ChunkDev& D, const std::vector<int>& lptr, const int* lidx, int lines,
                         int extent, int pass, int window_cap) {
  cudaStream_t s = stream_;
  int wmax = mixed_window_capacity(pass);
  if (window_cap >= 0) wmax = std::min(wmax, window_cap);
  const double split_min = window_cap >= 0 ? 0.0 : 0.5;
  // The outer sums stage their products in the block's warp buffers.
  const int round_cap = (kChunkThreads / 32) * kChunkCapF;
  ChunkPlan P = plan_chunks(lptr, lidx, lines, extent, kChunkCapF, wmax, num_sms_,
                            static_cast<int>(sizeof(float)), split_min, 0.999, round_cap);
  if (P.error) throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "chunk layout planning failed"};
  D.nrows = lines;
  D.split = P.split;
  D.nlong = static_cast<int>(P.longs.size());
  D.npieces = P.npieces;
  D.wmax = P.wmax;
  D.grid = P.grid;
  D.staged = P.staged;
  D.coverage = P.coverage;
  D.smem = mixed_step_smem(pass, P.wmax);
  D.chunks.upload(P.chunks.data(), P.chunks.size(), s);
  D.longs.upload(P.longs.data(), P.longs.size(), s);
  D.segs.upload(P.segs.data(), P.segs.size(), s);
  D.seg_start.upload(P.seg_start.data(), P.seg_start.size(), s);
  D.pieces.allocate(static_cast<size_t>(D.npieces) + 1);
  D.nmain = D.nouter = 0;
  if (P.split) {
    D.nmain = static_cast<long long>(P.idx.size());
    D.nouter = static_cast<long long>(P.oidx.size());
    D.ptr.upload_padded(P.ptr.data(), P.ptr.size(), kPad, s);
    D.idx.upload_padded(P.idx.data(), P.idx.size(), kPad, s);
    D.map.upload(P.map.data(), P.map.size(), s);
    D.optr.upload_padded(P.optr.data(), P.optr.size(), kPad, s);
    D.oidx.upload_padded(P.oidx.data(), P.oidx.size(), kPad, s);
    D.omap.upload(P.omap.data(), P.omap.size(), s);
    D.orounds.upload(P.orounds.data(), P.orounds.size(), s);
    D.oround_start.upload(P.oround_start.data(), P.oround_start.size(), s);
  } else {
    for (DeviceArray<int>* a : {&D.ptr, &D.idx, &D.map, &D.optr, &D.oidx, &D.omap}) a->release();
    D.orounds.release();
    D.oround_start.release();
  }
  D.fval.release();
  D.foval.release();
  D.fouter.release();
}

ChunkSet<float> Engine::chunk_set(const ChunkDev& D, const int* full_ptr, const int* full_idx,
                                  const float* full_val) const {
  ChunkSet<float> c{};
  c.chunks = D.chunks.ptr;
  c.segs = D.segs.ptr;
  c.seg_start = D.seg_start.ptr;
  c.longs = D.longs.ptr;
  c.nlong = D.nlong;
  c.npieces = D.npieces;
  c.nrows = D.nrows;
  c.wmax = D.wmax;
  if (D.split) {
    c.ptr = D.ptr.ptr;
    c.idx = D.idx.ptr;
    c.optr = D.optr.ptr;
    c.oidx = D.oidx.ptr;
    c.orounds = D.orounds.ptr;
    c.oround_start = D.oround_start.ptr;
    c.val = D.fval.ptr;
    c.oval = D.foval.ptr;
    c.outer = D.fouter.ptr;
  } else {
    c.ptr = full_ptr;
    c.idx = full_idx;
    c.val = full_val;
    c.outer = nullptr;
  }
  return c;
}

void Engine::fill_buffers() {
  const TileSet<double> csc{csc_ptr_.ptr,   csc_idx_.ptr, csc_s_.ptr,   csc_tiles_.ptr,
                            csc_longs_.ptr, ntiles_csc_,  nlong_csc_,   nchunks_csc_,
                            n_,             lanes_csc_};
  const TileSet<double> csr{csr_ptr_.ptr,   csr_idx_.ptr, csr_s_.ptr,   csr_tiles_.ptr,
                            csr_longs_.ptr, ntiles_csr_,  nlong_csr_,   nchunks_csr_,
                            m_,             lanes_csr_};
  StepBuffers& b = step_;
  b.ctl = ctl_.ptr;
  b.csc = csc;
  b.csr = csr;
  b.x[0] = x0_.ptr;
  b.x[1] = x1_.ptr;
  b.y[0] = y0_.ptr;
  b.y[1] = y1_.ptr;
  b.x_sum = x_sum_.ptr;
  b.y_sum = y_sum_.ptr;
  b.xd = xd_.ptr;
  b.c = cs_.ptr;
  b.l = ls_.ptr;
  b.u = us_.ptr;
  b.rl = rls_.ptr;
  b.ru = rus_.ptr;
  b.step_factors = step_factors_.ptr;
  b.step_factors_n = kStepFactorTable;
  b.part_primal = part_primal_.ptr;
  b.part_dual = part_dual_.ptr;
  b.chunk_primal = chunk_primal_.ptr;
  b.chunk_dual = chunk_dual_.ptr;
  b.csc.tile_win = step_csc_.tile_win.ptr;
  b.csc.windows = step_csc_.windows.ptr;
  b.csc.wmax = step_csc_.wmax;
  b.csr.tile_win = step_csr_.tile_win.ptr;
  b.csr.windows = step_csr_.windows.ptr;
  b.csr.wmax = step_csr_.wmax;
  b.grid_primal = step_csc_.grid;
  b.grid_dual = step_csr_.grid;
  b.smem_primal = step_csc_.smem;
  b.smem_dual = step_csr_.smem;

  EvalBuffers& e = eval_;
  e.ctl = ctl_.ptr;
  e.csc = csc;
  e.csc.val = csc_raw_.ptr;
  e.csr = csr;
  e.csr.val = csr_raw_.ptr;
  e.x[0] = x0_.ptr;
  e.x[1] = x1_.ptr;
  e.y[0] = y0_.ptr;
  e.y[1] = y1_.ptr;
  e.x_sum = x_sum_.ptr;
  e.y_sum = y_sum_.ptr;
  e.x_rst = x_rst_.ptr;
  e.y_rst = y_rst_.ptr;
  e.dr = dr_.ptr;
  e.dc = dc_.ptr;
  e.cost = cost_.ptr;
  e.col_cost = col_cost_.ptr;
  e.l = l_.ptr;
  e.u = u_.ptr;
  e.rl = rl_.ptr;
  e.ru = ru_.ptr;
  e.bound_norm = bound_norm_;
  e.cost_norm = cost_norm_;
  e.sense = sense_;
  e.xu[0] = xu0_.ptr;
  e.xu[1] = xu1_.ptr;
  e.yu[0] = yu0_.ptr;
  e.yu[1] = yu1_.ptr;
  e.reduced = reduced_.ptr;
  e.best_x = best_x_.ptr;
  e.best_y = best_y_.ptr;
  e.chunk_cols = chunk_cols_.ptr;
  e.chunk_rows = chunk_rows_.ptr;
  e.part_rows0 = part_rows0_.ptr;
  e.part_cols = part_cols_.ptr;
  e.part_rows1 = part_rows1_.ptr;
  e.grid_rows = grid_csr_;
  e.grid_cols = grid_csc_;
  e.m = m_;
  e.n = n_;
}

void Engine::precondition(long long seed) {
  (void)seed;
  cudaStream_t s = stream_;
  const size_t nb = static_cast<size_t>(nnz_) * sizeof(double);
  if (nnz_ > 0) {
    SGB_CUDA(cudaMemcpyAsync(csc_s_.ptr, csc_raw_.ptr, nb, cudaMemcpyDeviceToDevice, s));
    SGB_CUDA(cudaMemcpyAsync(csr_s_.ptr, csr_raw_.ptr, nb, cudaMemcpyDeviceToDevice, s));
  }
  launch_fill(dr_.ptr, m_, 1.0, s);
  launch_fill(dc_.ptr, n_, 1.0, s);
  for (int pass = 0; pass < 11; ++pass) {  // 10 Ruiz rounds, then Pock-Chambolle
    launch_scaling_round(m_, n_, step_.csr, step_.csc, csr_s_.ptr, csc_s_.ptr, row_acc_.ptr,
                         col_acc_.ptr, dr_.ptr, dc_.ptr, pass == 10 ? 1 : 0, s);
  }
  launch_scale_vectors(m_, n_, cost_.ptr, l_.ptr, u_.ptr, rl_.ptr, ru_.ptr, dr_.ptr, dc_.ptr,
                       cs_.ptr, ls_.ptr, us_.ptr, rls_.ptr, rus_.ptr, s);
  SGB_CUDA(cudaGetLastError());
  scaled_ = true;
}

// The FP32 scaled values of the split chunk layouts' main and outer parts, gathered from the
// full layouts' FP64 scaled values (each mixed solve, after the preconditioning).
void Engine::fill_split_values() {
  cudaStream_t s = stream_;
  const std::pair<ChunkDev*, const double*> layouts[] = {{&ck_csc_f_, csc_s_.ptr},
                                                          {&ck_csr_f_, csr_s_.ptr}};
  for (const auto& l : layouts) {
    ChunkDev& D = *l.first;
    if (!D.split) continue;
    launch_gather_values(l.second, D.map.ptr, D.fval.ptr, D.nmain, s);
    launch_gather_values(l.second, D.omap.ptr, D.foval.ptr, D.nouter, s);
  }
}

// src/la/scaling.cpp:161-194 on the device. The start vector is the reference's own
// std::mt19937(seed) + uniform_real_distribution(-1, 1) stream, drawn on the host.
double Engine::power_iteration(long long seed) {
  if (m_ == 0 || n_ == 0 || nnz_ == 0) return 1.0;
  cudaStream_t s = stream_;
  std::mt19937 rng(static_cast<unsigned>(seed) + 1u);
  std::uniform_real_distribution<double> spread(-1.0, 1.0);
  std::vector<double> v(static_cast<size_t>(n_));
  for (double& value : v) value = spread(rng);
  SGB_CUDA(cudaMemcpyAsync(power_v_.ptr, v.data(), v.size() * sizeof(double),
                           cudaMemcpyHostToDevice, s));
  const int iterations = 30;
  const int grid = std::min(num_sms_ * 4, std::max(1, (n_ + 255) / 256));
  double* norms = power_norms_.ptr;  // [2*step] = length^2, [2*step+1] = next
  for (int step = 0; step < iterations; ++step) {
    launch_sumsq(power_v_.ptr, n_, scalars_.ptr, norms + 2 * step, tickets_.ptr, s, grid);
    launch_scale_div(power_v_.ptr, n_, norms + 2 * step, s);
    launch_spmv(step_.csr, power_v_.ptr, power_av_.ptr, chunk_spmv_.ptr, tickets_.ptr + 1,
                product_error(), s, grid_csr_);
    launch_spmv(step_.csc, power_av_.ptr, power_v_.ptr, chunk_spmv_.ptr, tickets_.ptr + 1,
                product_error(), s, grid_csc_);
    launch_sumsq(power_v_.ptr, n_, scalars_.ptr, norms + 2 * step + 1, tickets_.ptr, s, grid);
  }
  SGB_CUDA(cudaGetLastError());
  std::vector<double> host(2 * iterations);
  SGB_CUDA(cudaMemcpyAsync(host.data(), norms, host.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, s));
  check_product_error();
  double norm = 0.0;
  for (int step = 0; step < iterations; ++step) {
    if (std::sqrt(host[2 * step]) == 0.0) return 1.0;
    norm = std::sqrt(std::sqrt(host[2 * step + 1]));
  }
  return norm > 0.0 ? norm * 1.01 : 1.0;
}

void Engine::scaling(long long seed, double* row_scale, double* col_scale, double* scaled_values,
                     double* spectral_norm) {
  require_loaded();
  SGB_CUDA(cudaSetDevice(device_));
  precondition(seed);
  const double norm = power_iteration(seed);
  cudaStream_t s = stream_;
  if (row_scale) SGB_CUDA(cudaMemcpyAsync(row_scale, dr_.ptr, m_ * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (col_scale) SGB_CUDA(cudaMemcpyAsync(col_scale, dc_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (scaled_values && nnz_ > 0) {
    SGB_CUDA(cudaMemcpyAsync(scaled_values, csc_s_.ptr, nnz_ * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  }
  SGB_CUDA(cudaStreamSynchronize(s));
  if (spectral_norm) *spectral_norm = norm;
}

void Engine::spmv(int op, int scaled, const double* in, double* out) {
  require_loaded();
  if (scaled && !scaled_) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no preconditioning has run yet"};
  }
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  const int in_len = op == 0 ? n_ : m_;
  const int out_len = op == 0 ? m_ : n_;
  DeviceArray<double> din, dout;
  din.upload(in, static_cast<size_t>(in_len), s);
  dout.allocate(static_cast<size_t>(out_len));
  TileSet<double> a = op == 0 ? step_.csr : step_.csc;
  if (!scaled) a.val = op == 0 ? csr_raw_.ptr : csc_raw_.ptr;
  launch_spmv(a, din.ptr, dout.ptr, chunk_spmv_.ptr, tickets_.ptr + 1, product_error(), s,
              op == 0 ? grid_csr_ : grid_csc_);
  SGB_CUDA(cudaGetLastError());
  if (out_len > 0) {
    SGB_CUDA(cudaMemcpyAsync(out, dout.ptr, out_len * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  check_product_error();
}

// The error word of the tile products (k_spmv), read at a synchronising point: it waits for
// the stream, and a product whose bounded wait gave up since the last check makes the call
// fail with a device error (the word is cleared for the next one).
void Engine::check_product_error() {
  unsigned int word = 0;
  SGB_CUDA(cudaMemcpyAsync(&word, product_error(), sizeof(word), cudaMemcpyDeviceToHost,
                           stream_));
  SGB_CUDA(cudaStreamSynchronize(stream_));
  if (product_error_status(word) != SANKHYA_GB300_OK) {
    SGB_CUDA(cudaMemsetAsync(product_error(), 0, sizeof(word), stream_));
    SGB_CUDA(cudaStreamSynchronize(stream_));
    throw EngineError{product_error_status(word), "a sparse product's tile copy did not complete "
                                                  "in time; its result was not used"};
  }
}

int product_error_status(unsigned int word) {
  return word == 0 ? SANKHYA_GB300_OK : SANKHYA_GB300_ERROR_DEVICE;
}

static_assert(kNoAllocMaxChunks == SANKHYA_GB300_NOALLOC_MAX_CHUNKS,
              "the header states the scratch size");

void Engine::spmv_noalloc(int op, int scaled, const double* in, double* out,
                          cudaStream_t stream) {
  require_loaded();
  if (op != 0 && op != 1) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, format("op must be 0 or 1, not %d", op)};
  }
  if (scaled && !scaled_) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no preconditioning has run yet"};
  }
  const int in_len = op == 0 ? n_ : m_;
  const int out_len = op == 0 ? m_ : n_;
  if ((in_len > 0 && in == nullptr) || (out_len > 0 && out == nullptr)) {
    throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "null device buffer"};
  }
  TileSet<double> a = op == 0 ? step_.csr : step_.csc;
  if (a.nchunks > kNoAllocMaxChunks) {
    throw EngineError{
        SANKHYA_GB300_ERROR_ARGUMENT,
        format("this matrix needs %d long-row chunk slots (one per %d entries of a row longer "
               "than %d); the allocation-free product holds at most %d",
               a.nchunks, kCap, kCap, kNoAllocMaxChunks)};
  }
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream != nullptr ? stream : stream_;
  double* chunks = nullptr;
  unsigned int* ticket = nullptr;
  unsigned int* error = nullptr;
  SGB_CUDA(noalloc_scratch(device_, s, &chunks, &ticket, &error));
  if (!scaled) a.val = op == 0 ? csr_raw_.ptr : csc_raw_.ptr;
  launch_spmv(a, in, out, chunks, ticket, error, s, op == 0 ? grid_csr_ : grid_csc_);
  SGB_CUDA(cudaGetLastError());
}

void Engine::init_iterates(const sankhya_gb300_params& p) {
  cudaStream_t s = stream_;
  launch_project_start(n_, ls_.ptr, us_.ptr, x0_.ptr, s);
  launch_fill(y0_.ptr, m_, 0.0, s);
  launch_fill(x_sum_.ptr, n_, 0.0, s);
  launch_fill(y_sum_.ptr, m_, 0.0, s);
  launch_fill(y_rst_.ptr, m_, 0.0, s);
  launch_fill(best_y_.ptr, m_, 0.0, s);
  if (n_ > 0) {
    SGB_CUDA(cudaMemcpyAsync(x_rst_.ptr, x0_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    // best_x starts as the SCALED start point, as the reference's does (pdhg.cpp:190).
    SGB_CUDA(cudaMemcpyAsync(best_x_.ptr, x0_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  (void)p;
}

void Engine::build_graphs(int steps) {
  if (graph_steps_ == steps && graph_exec_[0] != nullptr) return;
  destroy_graphs();
  for (int slot = 0; slot < 2; ++slot) {
    cudaGraph_t graph = nullptr;
    SGB_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; ++k) {
      launch_pdhg_step(step_, stream_);
      if ((k + 1) % kEvalStride == 0 || k + 1 == steps) launch_evaluation(eval_, stream_);
    }
    cudaMemcpyAsync(snapshot_ + slot, ctl_.ptr, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_);
    const cudaError_t end = cudaStreamEndCapture(stream_, &graph);
    SGB_CUDA(end);
    const cudaError_t inst = cudaGraphInstantiate(&graph_exec_[slot], graph, 0);
    cudaGraphDestroy(graph);
    SGB_CUDA(inst);
  }
  graph_steps_ = steps;
}

void Engine::run_graphs(const sankhya_gb300_params& p, double t0, cudaGraphExec_t* graphs,
                        Ctl* snapshot, bool forward_log, long long iteration_offset,
                        int* stop_status) {
  Trace trace("pdhg iterations");
  const bool has_time_limit = p.time_limit < 1e300;
  long long logged = 0;
  auto launch = [&](int slot) {
    ++graphs_launched_;
    SGB_CUDA(cudaGraphLaunch(graphs[slot], stream_));
    SGB_CUDA(cudaEventRecord(done_event_[slot], stream_));
  };
  // The time limit is checked before any step, as the reference's loop does.
  if (has_time_limit && (p.time_limit <= 0.0 || now_seconds() - t0 > p.time_limit)) {
    *stop_status = SANKHYA_GB300_TIME_LIMIT;
    return;
  }
  launch(0);
  launch(1);
  for (long long k = 0;; ++k) {
    const int slot = static_cast<int>(k & 1);
    SGB_CUDA(cudaEventSynchronize(done_event_[slot]));
    const Ctl& snap = snapshot[slot];
    if (forward_log && p.log != nullptr && snap.log_count > logged) {
      const double elapsed = now_seconds() - t0;
      const long long first = std::max(logged, snap.log_count - kLogRing);
      for (long long r = first; r < snap.log_count; ++r) {
        const EvalRecord& rec = snap.log[r % kLogRing];
        p.log(p.log_user, iteration_offset + rec.iteration,
              sense_ * rec.primal_objective + offset_, rec.primal, rec.dual, elapsed);
      }
      logged = snap.log_count;
    }
    if (snap.done != kRunning) break;
    if (has_time_limit && now_seconds() - t0 > p.time_limit) {
      *stop_status = SANKHYA_GB300_TIME_LIMIT;
      break;
    }
    if ((p.interrupt != nullptr && *p.interrupt != 0) ||
        (p.poll != nullptr &&
         p.poll(p.poll_user, iteration_offset + snap.iteration,
                sense_ * snap.best.primal_objective + offset_) != 0)) {
      *stop_status = SANKHYA_GB300_INTERRUPTED;
      break;
    }
    launch(slot);
  }
  SGB_CUDA(cudaStreamSynchronize(stream_));
}

void Engine::final_evaluation() {
  // final_mode = 1: the evaluation kernels evaluate (best_x, best_y) only.
  const int one = 1;
  SGB_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(ctl_.ptr) + offsetof(Ctl, final_mode), &one,
                           sizeof(int), cudaMemcpyHostToDevice, stream_));
  launch_evaluation(eval_, stream_);
  SGB_CUDA(cudaGetLastError());
}

// Device preconditioning, the spectral-norm estimate and the scaled entry range (the log
// line of src/pdhg/pdhg.cpp:132-133); the same for both precisions.
void Engine::setup(const sankhya_gb300_params& p, sankhya_gb300_result* r, double* norm) {
  Trace trace("pdhg scaling");
  cudaStream_t s = stream_;
  precondition(p.random_seed);
  *norm = power_iteration(p.random_seed);
  const int grid = std::min(num_sms_ * 4, std::max(1, static_cast<int>((nnz_ + 255) / 256)));
  launch_abs_minmax(csc_s_.ptr, static_cast<int>(nnz_), scalars_.ptr,
                    scalars_.ptr + 2 * grid + 2, tickets_.ptr, s, grid);
  double mm[2] = {0.0, 0.0};
  SGB_CUDA(cudaMemcpyAsync(mm, scalars_.ptr + 2 * grid + 2, 2 * sizeof(double),
                           cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  r->scaled_max_abs = mm[0];
  r->scaled_min_abs = mm[1];
  r->spectral_norm = *norm;
}

void Engine::solve(const sankhya_gb300_params& p, sankhya_gb300_result* r) {
  require_loaded();
  Trace trace(p.precision == SANKHYA_GB300_MIXED ? "pdhg solve (mixed)" : "pdhg solve");
  const double t0 = now_seconds();
  std::memset(r, 0, sizeof(*r));
  if (p.precision != SANKHYA_GB300_FP64 && p.precision != SANKHYA_GB300_MIXED) {
    throw EngineError{SANKHYA_GB300_ERROR_OPTION, "pdhg_precision must be fp64 or mixed"};
  }
  SGB_CUDA(cudaSetDevice(device_));
  SGB_CUDA(cudaEventRecord(timing_[0], stream_));
  graphs_launched_ = 0;
  extra_launches_ = 0;
  if (p.precision == SANKHYA_GB300_MIXED) {
    solve_mixed(p, r, t0);
  } else {
    solve_fp64(p, r, t0);
  }
  last_precision_ = p.precision;
  solved_ = true;
  r->solve_seconds = now_seconds() - t0;
}

void Engine::report(const sankhya_gb300_params& p, const Ctl& c, bool converged,
                    long long iterations, long long restarts, int stop_status,
                    sankhya_gb300_result* r) {
  const Residuals& f = c.final_residuals;
  r->final_residuals = sankhya_gb300_residuals{f.primal,          f.dual,           f.gap,
                                              f.primal_objective, f.dual_objective,
                                              f.absolute_primal,  f.absolute_dual,
                                              f.gap_as_verified,  f.complementarity};
  r->converged = converged;
  // src/pdhg/pdhg.cpp:506-557: `optimal` only for a point that meets the project standard.
  const bool verifiable = converged && meets_project_standard(f);
  std::string message;
  if (verifiable) {
    r->status = SANKHYA_GB300_OPTIMAL;
    message = format(
        "converged after %lld iterations and %lld restarts; absolute primal %.3e, dual %.3e, "
        "relative gap %.3e",
        iterations, restarts, f.absolute_primal, f.absolute_dual, f.gap_as_verified);
  } else if (converged) {
    r->status = SANKHYA_GB300_FEASIBLE;
    message = format(
        "met the requested relative tolerance %.1e after %lld iterations, but NOT the absolute "
        "standard this project verifies against (primal %.3e vs 1.0e-07, dual %.3e vs 1.0e-07, "
        "relative gap %.3e vs 1.0e-09). Reported as feasible, not optimal. %s",
        p.tolerance, iterations, f.absolute_primal, f.absolute_dual, f.gap_as_verified,
        p.stop_at_request ? "pdhg_stop_at_request is on, so this is the cheap answer that was "
                            "asked for; turn it off to run on to the standard"
                          : "Tighten --option pdhg_tolerance to close it");
  } else {
    r->status = stop_status == SANKHYA_GB300_TIME_LIMIT || stop_status == SANKHYA_GB300_INTERRUPTED
                    ? stop_status
                    : SANKHYA_GB300_ITERATION_LIMIT;
    message = format(
        "stopped at relative primal %.3e, dual %.3e, gap %.3e after %lld iterations and %lld "
        "restarts (target %.1e)",
        f.primal, f.dual, f.gap, iterations, restarts, p.tolerance);
  }
  r->dual_bound = verifiable ? sense_ * f.dual_objective + offset_
                             : (sense_ < 0.0 ? std::numeric_limits<double>::infinity()
                                             : -std::numeric_limits<double>::infinity());
  r->objective = offset_ + c.model_objective;
  std::snprintf(r->message, sizeof(r->message), "%s", message.c_str());
}

void Engine::solve_fp64(const sankhya_gb300_params& p, sankhya_gb300_result* r, double t0) {
  cudaStream_t s = stream_;
  const long long launches_before = kernel_launch_count();
  double norm = 1.0;
  setup(p, r, &norm);
  init_iterates(p);

  Ctl c;
  std::memset(&c, 0, sizeof(c));
  c.eta = norm > 0.0 ? 1.0 / norm : 1.0;
  c.omega = 1.0;
  c.spectral_norm = norm;
  c.eta_ceiling = 1.0e3 / std::max(norm, 1e-12);
  c.restart_kkt = std::numeric_limits<double>::infinity();
  c.tolerance = p.tolerance;
  c.iteration_limit = p.iteration_limit < 0 ? 1000000 : p.iteration_limit;
  c.use_restarts = p.restart != 0;
  c.stop_at_request = p.stop_at_request != 0;
  c.stop_rule = p.stop_rule == SANKHYA_GB300_STOP_RELATIVE ? 1 : 0;
  c.best.primal = c.best.dual = c.best.gap = std::numeric_limits<double>::infinity();
  SGB_CUDA(cudaMemcpyAsync(ctl_.ptr, &c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  const double t_loop = now_seconds();
  r->setup_seconds = t_loop - t0;

  int stop_status = SANKHYA_GB300_ITERATION_LIMIT;
  const long long launches_setup = kernel_launch_count() - launches_before;
  build_graphs(p.steps_per_poll > 0 ? p.steps_per_poll : 32);  // capture launches nothing
  const long long count_after_capture = kernel_launch_count();
  run_graphs(p, t0, graph_exec_, snapshot_, true, 0, &stop_status);
  const double t_end_loop = now_seconds();
  final_evaluation();
  SGB_CUDA(cudaEventRecord(timing_[1], s));
  SGB_CUDA(cudaMemcpyAsync(&c, ctl_.ptr, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  r->loop_seconds = t_end_loop - t_loop;
  float device_ms = 0.0f;
  SGB_CUDA(cudaEventElapsedTime(&device_ms, timing_[0], timing_[1]));
  r->device_seconds = 1e-3 * device_ms;
  launches_ = launches_setup + (kernel_launch_count() - count_after_capture) +
              graphs_launched_ * graph_kernel_launches(graph_steps_);
  r->kernel_launches = launches_;
  r->staged_fraction[0] = step_csc_.staged;
  r->staged_fraction[1] = step_csr_.staged;
  if (c.error) {
    throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "a tile copy did not complete in time"};
  }
  r->iterations = c.iteration;
  r->attempts = c.attempts;
  r->restarts = c.restarts;
  r->evaluations = c.evaluations;
  report(p, c, c.done == kConverged, c.iteration, c.restarts, stop_status, r);
}

// The mixed method (mixed.cuh): FP32 inner PDHG on correction problems, FP64 anchor updates,
// and the reference's exact FP64 evaluation after every round.
void Engine::solve_mixed(const sankhya_gb300_params& p, sankhya_gb300_result* r, double t0) {
  cudaStream_t s = stream_;
  allocate_mixed();
  const long long launches_before = kernel_launch_count();
  double norm = 1.0;
  setup(p, r, &norm);
  // FP32 copies of the scaled values; the FP64 anchor starts at proj(0), y = 0.
  launch_to_float(csc_s_.ptr, csc_f_.ptr, nnz_, s);
  launch_to_float(csr_s_.ptr, csr_f_.ptr, nnz_, s);
  launch_to_float(cs_.ptr, csf_.ptr, n_, s);
  extra_launches_ += 3;
  fill_split_values();
  launch_project_start(n_, ls_.ptr, us_.ptr, anchor_x_.ptr, s);
  launch_fill(anchor_y_.ptr, m_, 0.0, s);
  extra_launches_ += 2;
  {
    // The scaled problem's norms, for the inner loop's relative residuals.
    std::vector<double> h(static_cast<size_t>(std::max(m_, n_)));
    double bs = 0.0, cs2 = 0.0;
    std::vector<double> rl(static_cast<size_t>(m_)), ru(static_cast<size_t>(m_));
    if (m_ > 0) {
      SGB_CUDA(cudaMemcpyAsync(rl.data(), rls_.ptr, m_ * sizeof(double), cudaMemcpyDeviceToHost, s));
      SGB_CUDA(cudaMemcpyAsync(ru.data(), rus_.ptr, m_ * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    if (n_ > 0) {
      SGB_CUDA(cudaMemcpyAsync(h.data(), cs_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    SGB_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < m_; ++i) {
      const double b = !std::isinf(rl[i]) ? rl[i] : (!std::isinf(ru[i]) ? ru[i] : 0.0);
      bs += b * b;
    }
    for (int j = 0; j < n_; ++j) cs2 += h[j] * h[j];
    bound_norm_s_ = std::sqrt(bs);
    cost_norm_s_ = std::sqrt(cs2);
  }
  const double t_loop = now_seconds();
  r->setup_seconds = t_loop - t0;
  const long long launches_setup = kernel_launch_count() - launches_before;

  const int steps = p.steps_per_poll > 0 ? p.steps_per_poll : 32;
  build_mixed_graphs(steps);
  const long long limit = p.iteration_limit < 0 ? 1000000 : p.iteration_limit;
  const double inf = std::numeric_limits<double>::infinity();
  const int rgrid = std::min(num_sms_ * 4, std::max(1, (std::max(m_, n_) + 255) / 256));
  RoundBuffers rb{};
  rb.ctl = ctl_mixed_.ptr;
  rb.m = m_;
  rb.n = n_;
  rb.cs = cs_.ptr;
  rb.ls = ls_.ptr;
  rb.us = us_.ptr;
  rb.rls = rls_.ptr;
  rb.rus = rus_.ptr;
  rb.dr = dr_.ptr;
  rb.dc = dc_.ptr;
  rb.xbar = anchor_x_.ptr;
  rb.ybar = anchor_y_.ptr;
  rb.ax = ax64_.ptr;
  rb.aty = aty64_.ptr;
  rb.cf = cf_.ptr;
  rb.lf = lf_.ptr;
  rb.uf = uf_.ptr;
  rb.gu = gu_.ptr;
  rb.gl = gl_.ptr;
  rb.yhat = yhat_.ptr;
  rb.u_src = ubest_.ptr;
  rb.v_src = vbest_.ptr;
  rb.best_x = best_x_.ptr;
  rb.best_y = best_y_.ptr;
  rb.part = scalars_.ptr;
  rb.out = power_norms_.ptr;
  rb.ticket = tickets_.ptr + 2;
  rb.grid = rgrid;

  // FP64 control block for the exact evaluations.
  Ctl fc;
  std::memset(&fc, 0, sizeof(fc));
  fc.final_mode = 1;
  SGB_CUDA(cudaMemcpyAsync(ctl_.ptr, &fc, sizeof(Ctl), cudaMemcpyHostToDevice, s));

  // The inner loop's state carries across rounds: a round is only a change of variables, so
  // the step size, primal weight, restart bookkeeping and the GLOBAL iteration count go on
  // as one PDHG run. A round ends at each restart the inner loop decides (the anchor moves to
  // the current iterate -- the restart point -- and the correction is rescaled to the new
  // residuals), or when the inner KKT estimate meets the round's target (the anchor moves to
  // the better candidate and is checked exactly), or at a limit.
  Ctl c;
  std::memset(&c, 0, sizeof(c));
  c.eta = norm > 0.0 ? 1.0 / norm : 1.0;
  c.omega = 1.0;
  c.spectral_norm = norm;
  c.eta_ceiling = 1.0e3 / std::max(norm, 1e-12);
  c.restart_kkt = inf;
  c.tolerance = p.tolerance;
  c.iteration_limit = limit;
  c.use_restarts = p.restart != 0;
  c.inner_mode = 1;
  c.bound_norm_s = bound_norm_s_;
  c.cost_norm_s = cost_norm_s_;
  double dp = 1.0, dd = 1.0;
  double target = 0.5 * p.tolerance;
  long long rounds = 0;
  int stop_status = SANKHYA_GB300_ITERATION_LIMIT;
  bool converged = false;
  Ctl exact_ctl;
  std::memset(&exact_ctl, 0, sizeof(exact_ctl));
  const auto stop_test = [&](const Residuals& f) {
    return p.stop_rule == SANKHYA_GB300_STOP_RELATIVE
               ? worst(f) <= p.tolerance
               : meets_request(f, p.tolerance) &&
                     (p.stop_at_request != 0 || meets_project_standard(f));
  };
  for (;; ++rounds) {
    // Anchor residuals in FP64, then the scales of this round's correction problem.
    launch_spmv(step_.csr, anchor_x_.ptr, ax64_.ptr, chunk_spmv_.ptr, tickets_.ptr + 1,
                product_error(), s, grid_csr_);
    launch_spmv(step_.csc, anchor_y_.ptr, aty64_.ptr, chunk_spmv_.ptr, tickets_.ptr + 1,
                product_error(), s, grid_csc_);
    launch_round_measure(rb, s);
    extra_launches_ += 3;
    double out[3];
    SGB_CUDA(cudaMemcpyAsync(out, rb.out, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    check_product_error();
    // 1 / residual, never below 1, at most 1e3 times the previous scale and 1e15 overall: an
    // anchor whose residual is exactly zero must not push the FP32 data out of range.
    const auto scale = [&](double residual, double prev) {
      if (rounds == 0) return 1.0;
      const double want = 1.0 / std::max(residual, 1e-300);
      return std::max(1.0, std::min({want, prev * 1e3, 1e15}));
    };
    const double dp_new = scale(out[0], dp);
    const double dd_new = scale(out[1], dd);
    // The primal weight lives in correction units: omega_c = omega (Dd / Dp).
    c.omega = std::min(std::max(c.omega * (dd_new / dd) / (dp_new / dp), 1e-10), 1e10);
    dp = dp_new;
    dd = dd_new;
    c.dp = dp;
    c.dd = dd;
    c.pobj0 = out[2];
    c.round_target = target;
    c.cur = 0;
    c.averaged = 0;
    c.pending_add = 0;
    c.done = kRunning;
    c.eval_now = c.copy_best = c.do_restart = 0;
    c.best.primal = c.best.dual = c.best.gap = inf;
    std::memset(c.ticket, 0, sizeof(c.ticket));
    SGB_CUDA(cudaMemcpyAsync(ctl_mixed_.ptr, &c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    launch_round_build(rb, s);
    for (DeviceArray<float>* a : {&u0f_, &usumf_, &urstf_, &ubest_}) launch_fill_float(a->ptr, n_, 0.0f, s);
    for (DeviceArray<float>* a : {&v0f_, &vsumf_, &vrstf_, &vbest_, &auf0_}) {
      launch_fill_float(a->ptr, m_, 0.0f, s);
    }
    extra_launches_ += 10;
    SGB_CUDA(cudaGetLastError());
    int round_stop = SANKHYA_GB300_ITERATION_LIMIT;
    run_graphs(p, t0, mgraph_exec_, snapshot_mixed_, false, 0, &round_stop);
    SGB_CUDA(cudaMemcpyAsync(&c, ctl_mixed_.ptr, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    SGB_CUDA(cudaStreamSynchronize(s));
    if (c.error) {
      throw EngineError{SANKHYA_GB300_ERROR_DEVICE, "a tile copy did not complete in time"};
    }
    // A restart moves the anchor to the current iterate (the restart point); otherwise to
    // the better of the last evaluated candidates.
    if (c.done == kRestartRound) {
      rb.u_src = c.cur ? u1f_.ptr : u0f_.ptr;
      rb.v_src = c.cur ? v1f_.ptr : v0f_.ptr;
    } else {
      rb.u_src = ubest_.ptr;
      rb.v_src = vbest_.ptr;
    }
    launch_round_update(rb, s);
    final_evaluation();
    extra_launches_ += 5;
    SGB_CUDA(cudaMemcpyAsync(&exact_ctl, ctl_.ptr, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    SGB_CUDA(cudaStreamSynchronize(s));
    const Residuals& f = exact_ctl.final_residuals;
    if (p.log != nullptr) {
      p.log(p.log_user, c.iteration, sense_ * f.primal_objective + offset_, f.primal, f.dual,
            now_seconds() - t0);
    }
    if (stop_test(f)) {
      converged = true;
      break;
    }
    if (round_stop != SANKHYA_GB300_ITERATION_LIMIT) {
      stop_status = round_stop;
      break;
    }
    if (c.done == kIterationLimit || c.iteration >= limit) break;
    if (c.done == kConverged) {
      // The estimate met the target but the exact check did not: tighten the estimate's bar.
      target *= 0.3;
    }
  }
  const long long total_it = c.iteration, total_att = c.attempts, restarts = c.restarts;
  const long long evals = c.evaluations;
  SGB_CUDA(cudaEventRecord(timing_[1], s));
  SGB_CUDA(cudaStreamSynchronize(s));
  const double t_end_loop = now_seconds();
  r->loop_seconds = t_end_loop - t_loop;
  float device_ms = 0.0f;
  SGB_CUDA(cudaEventElapsedTime(&device_ms, timing_[0], timing_[1]));
  r->device_seconds = 1e-3 * device_ms;
  launches_ = launches_setup + extra_launches_ +
              graphs_launched_ * graph_kernel_launches(mgraph_steps_);
  r->kernel_launches = launches_;
  r->staged_fraction[0] = ck_csc_f_.staged;
  r->staged_fraction[1] = ck_csr_f_.staged;
  r->iterations = total_it;
  r->attempts = total_att;
  r->restarts = restarts;
  r->evaluations = evals;
  r->refinements = rounds + 1;
  report(p, exact_ctl, converged, total_it, restarts, stop_status, r);
}

void Engine::time_kernels(int reps, double* ms) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  // The kernels of the last solve's method, on its own control block (the FP32 pair for a
  // mixed solve, the FP64 pair otherwise).
  const bool mixed = last_precision_ == SANKHYA_GB300_MIXED;
  Ctl* ctl = mixed ? ctl_mixed_.ptr : ctl_.ptr;
  Ctl saved;
  SGB_CUDA(cudaMemcpyAsync(&saved, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  Ctl run = saved;
  run.done = kRunning;
  run.final_mode = 0;
  run.eval_now = 0;
  run.iteration_limit = std::numeric_limits<long long>::max();
  SGB_CUDA(cudaMemcpyAsync(ctl, &run, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  std::vector<cudaEvent_t> ev(3 * static_cast<size_t>(reps));
  for (auto& e : ev) SGB_CUDA(cudaEventCreate(&e));
  for (int r = 0; r < reps; ++r) {
    SGB_CUDA(cudaEventRecord(ev[3 * r], s));
    if (mixed) launch_mixed_primal(mixed_, s); else launch_primal_pass(step_, s);
    SGB_CUDA(cudaEventRecord(ev[3 * r + 1], s));
    if (mixed) launch_mixed_dual(mixed_, s); else launch_dual_pass(step_, s);
    SGB_CUDA(cudaEventRecord(ev[3 * r + 2], s));
  }
  SGB_CUDA(cudaGetLastError());
  SGB_CUDA(cudaStreamSynchronize(s));
  double primal = 0.0, dual = 0.0;
  for (int r = 0; r < reps; ++r) {
    float a = 0.0f, b = 0.0f;
    SGB_CUDA(cudaEventElapsedTime(&a, ev[3 * r], ev[3 * r + 1]));
    SGB_CUDA(cudaEventElapsedTime(&b, ev[3 * r + 1], ev[3 * r + 2]));
    primal += a;
    dual += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  SGB_CUDA(cudaMemcpyAsync(ctl, &saved, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  SGB_CUDA(cudaStreamSynchronize(s));
  ms[0] = primal / reps;
  ms[1] = dual / reps;
}

void Engine::solution(double* col_value, double* col_dual, double* row_dual) {
  require_loaded();
  if (!solved_) throw EngineError{SANKHYA_GB300_ERROR_ARGUMENT, "no solve has run"};
  SGB_CUDA(cudaSetDevice(device_));
  cudaStream_t s = stream_;
  std::vector<double> red, by;
  if (col_value && n_ > 0) {
    SGB_CUDA(cudaMemcpyAsync(col_value, best_x_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (col_dual && n_ > 0) {
    red.resize(static_cast<size_t>(n_));
    SGB_CUDA(cudaMemcpyAsync(red.data(), reduced_.ptr, n_ * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (row_dual && m_ > 0) {
    by.resize(static_cast<size_t>(m_));
    SGB_CUDA(cudaMemcpyAsync(by.data(), best_y_.ptr, m_ * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  SGB_CUDA(cudaStreamSynchronize(s));
  if (col_dual) {
    for (int j = 0; j < n_; ++j) col_dual[j] = sense_ * red[j];
  }
  if (row_dual) {
    for (int i = 0; i < m_; ++i) row_dual[i] = sense_ * (-by[i]);
  }
}

}  // namespace sgb

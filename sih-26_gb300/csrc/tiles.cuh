// tiles.cuh -- TMA-staged row tiles: the sparse-product engine under every pass.
//
// A TILE is a run of consecutive rows (of the CSR copy, or columns of the CSC copy) whose
// nonzeros fit one shared-memory buffer (kCap entries). A row longer than kCap is cut into
// CHUNK tiles of at most kCap entries. Block b of a grid of G owns the contiguous tile range
// [b T / G, (b + 1) T / G), so every sum below is taken in a fixed order (a run is
// bit-reproducible) and a block's gathers stay inside a narrow band of the vector wherever
// the matrix has block or banded structure.
//
// Each block runs an NB-stage pipeline over its tiles: thread 0 keeps NB - 1 bulk async
// copies (cp.async.bulk, the TMA engine's 1-D form) of the next tiles' index and value
// ranges in flight, each completing on its own mbarrier, while all threads work on the
// current tile. Working on a tile: `lanes` threads share a row, walk it in ascending index
// order reading (index, value) from shared memory, gather the vector entries and accumulate
// with FMA. A chunk tile is walked by all threads and reduced across the block into a
// per-chunk partial; the chunks of a long row are combined in chunk order by the last block
// of the kernel.
//
// WINDOWS. Random gathers from L2 are limited by sector requests (about one per clock per
// SM), far below HBM streaming speed. So the gathered vector is staged: at load time every
// tile gets the index range [lo, lo + len) that holds most of its entries (tiles in a row
// share one range, see build_windows), and a kernel with a Window copies that slice of the
// vector into shared memory with one bulk copy whenever the range changes. Entries inside
// it are gathered from shared memory (a few cycles per warp), the rest from global memory.
//
// Copies must start on 16 bytes and move a multiple of 16 bytes, so a tile's range is
// widened to multiples of 4 entries on both sides; the device arrays carry kPad entries of
// padding so the widened range never leaves the allocation (window ranges are multiples of
// 4 elements and gathered vectors carry kPad elements of padding too). Every mbarrier wait
// is bounded: a wait that gives up records an error in the control block, waits (bounded)
// for the block's copies still in flight, and the kernel returns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace sgb {

constexpr int kCap = 2048;        // entries per tile buffer
constexpr int kSlack = 8;         // widening of a tile range to 16-byte boundaries
constexpr int kPad = 8;           // padding entries at the end of every index / value array
constexpr int kTileThreads = 256;  // consumer threads of the FP64 tile blocks
constexpr int kBlockThreads = kTileThreads + 32;  // plus the producer warp
constexpr int kWideThreads = 512;  // consumer threads of the FP32 tile blocks
constexpr int kWideBlockThreads = kWideThreads + 32;
constexpr int kMaxTileRows = 256;  // rows of a tile, whatever the block size
// A row longer than this, in a layout of one lane per row, gets a tile of its own that one
// consumer warp sums (a WARP ROW): one thread walking a row of hundreds or thousands of
// dependent gathers holds up its whole block (the load-balance failure of long rows).
constexpr int kWarpRowMin = 64;
constexpr long long kWaitLimit = 1LL << 24;

struct Tile {
  int r0, r1;  // rows [r0, r1); r1 < 0 marks a chunk tile whose chunk slot is -r1 - 1
  int k0, k1;  // nonzeros [k0, k1)
};

struct LongRow {
  int row;
  int chunk0;   // first chunk slot
  int nchunks;
};

template <typename V>
struct TileSet {
  const int* ptr;       // nrows + 1
  const int* idx;       // nnz (+ kPad)
  const V* val;         // nnz (+ kPad)
  const Tile* tiles;
  const LongRow* longs;
  int ntiles;
  int nlong;
  int nchunks;
  int nrows;
  int lanes;            // threads per row inside a short tile (power of two, <= 32); a tile
                        // holds at most min(kMaxTileRows, threads / lanes) rows
  const int* tile_win;  // per tile: index into `windows`, or -1 (gathers from global memory)
  const int2* windows;  // {lo, len}: lo and len multiples of 4, len <= wmax
  int wmax;             // window capacity in gathered elements (0: this layout has none)
};

// A tile range's bounds: block b of G owns tiles [first, last).
__device__ __forceinline__ void block_tile_range(int ntiles, int& first, int& last) {
  const long long T = ntiles, G = gridDim.x, b = blockIdx.x;
  first = static_cast<int>((b * T) / G);
  last = static_cast<int>(((b + 1) * T) / G);
}

// Lanes per row for the FP32 layouts (the FP64 layouts use one lane per row, which sums
// each row in the reference's order): the smallest power of two for which a tile has at
// most kMaxTileRows rows and threads / lanes rows of average length fill at most two
// buffers. The tile is then cut at kCap entries with at least half of the threads busy.
// Asking instead that the rows fill only one buffer (every thread busy) gives tiles half as
// long, and on the 1M x 2M block-angular LP the column pass (avg 10 entries: 2 lanes against
// 4) measured 27% slower and the row pass (avg 20: 4 lanes against 8) 14% slower that way:
// each bulk copy in flight carries less of the matrix. One lane fewer again (2 for the
// rows) measured slower too.
inline int wide_lanes(double avg, int threads) {
  int lanes = 1;
  while (lanes < 32 && ((static_cast<double>(threads) / lanes) * avg > 2.0 * kCap ||
                        threads / lanes > kMaxTileRows)) {
    lanes *= 2;
  }
  return lanes;
}


// Host: the dynamic shared memory a kernel may still take on this device (the opt-in
// per-block limit less its static shared memory), and the window capacity (gathered
// elements, a multiple of 1024) left beside a pipeline of `pipe_bytes`.
inline int max_dynamic_smem(const void* kernel) {
  int dev = 0, optin = 0;
  cudaFuncAttributes attr{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
          cudaSuccess ||
      cudaFuncGetAttributes(&attr, kernel) != cudaSuccess) {
    cudaGetLastError();
    return 48 * 1024;
  }
  return optin - static_cast<int>(attr.sharedSizeBytes);
}

inline int window_bytes(int wmax, int elem_bytes) {
  return (wmax * elem_bytes + 127) & ~127;
}

inline int window_capacity(const void* kernel, int pipe_bytes, int elem_bytes) {
  const int budget = max_dynamic_smem(kernel) - pipe_bytes - 128;
  return budget > 0 ? (budget / elem_bytes) & ~1023 : 0;
}

// ---- PTX wrappers (mbarrier, bulk async copy) ---------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses to shared memory before later
// async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase; false if it did not complete within kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  long long spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins > kWaitLimit) return false;
  }
  return true;
}

// ---- The pipeline --------------------------------------------------------------------------

// A bounded wait that also gives up as soon as another thread has recorded an abort.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity,
                                                   volatile int* abort_flag) {
  long long spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins > kWaitLimit || *abort_flag) return false;
  }
  return true;
}

// NB tile buffers filled by a PRODUCER warp (the block's last warp; its lane 0 issues the bulk
// copies) and drained by CT / 32 CONSUMER warps. Buffer b has a FULL barrier (the
// producer's expect-tx arrival plus the copied bytes) and an EMPTY barrier (one arrival per
// consumer warp once it has finished with the tile). The consumer warps never wait for one
// another, only for data, so one warp's stall on a global gather overlaps the others' work.
//
// NR > 0 also stages, with each row tile, the slices [r0, r1) of NR per-row vectors of type
// V (the epilogue's operands: iterate, cost or bounds, running sum, ...), and every row tile
// brings its row pointers, so the consumers touch global memory only for gathers that fall
// outside a staged window and for the epilogue's stores.
constexpr int kRowStride = kMaxTileRows + 8;  // a tile's rows widened to 4-element bounds

template <typename V, int NB = 2, int NR = 0, int CT = kTileThreads>
struct TilePipe {
  static constexpr int kConsumers = CT;        // consumer threads (threads [0, CT))
  static constexpr int kConsumerWarps = CT / 32;
  static constexpr int kThreads = CT + 32;     // the block: consumers and the producer warp
  // Buffer b's entries start at idx0 + b * kStride / val0 + b * kStride (computed, never an
  // array indexed by b, so the pointers stay in registers).
  static constexpr int kStride = kCap + kSlack;
  static constexpr int kBuffers = NB;
  static constexpr int kRows = NR;
  static constexpr int kMeta = 8;  // ints per buffer: the Tile record and its window id
  static constexpr int kBars = 2 * NB + 2;
  int* idx0;
  V* val0;
  V* row0;        // NB x NR x kRowStride staged row values
  int* ptr0;      // NB x kRowStride staged row pointers
  int* meta0;     // NB x kMeta
  uint64_t* bar;  // full[NB], empty[NB], window release, window full
  const V* rsrc[NR > 0 ? NR : 1];  // the per-row vectors (global memory)
  const V* cur_rows;  // staged rows of the current tile
  int row_base;       // the row cur_rows[0] holds (the tile's first row rounded down to 4)
  bool rows_staged;   // false: row() reads global memory (long rows, finished after the tiles)

  // Dynamic shared memory of the pipeline; a staged window (Window below) follows it.
  __host__ __device__ static constexpr int bytes() {
    return (NB * kStride * static_cast<int>(sizeof(int) + sizeof(V)) +
            NB * NR * kRowStride * static_cast<int>(sizeof(V)) +
            NB * (kRowStride + kMeta) * static_cast<int>(sizeof(int)) + 8 * kBars + 127) &
           ~127;
  }

  __device__ __forceinline__ int* idx(int b) const { return idx0 + b * kStride; }
  __device__ __forceinline__ V* val(int b) const { return val0 + b * kStride; }
  __device__ __forceinline__ V* rows(int b) const { return row0 + b * NR * kRowStride; }
  __device__ __forceinline__ int* ptrs(int b) const { return ptr0 + b * kRowStride; }
  __device__ __forceinline__ int* meta(int b) const { return meta0 + b * kMeta; }
  __device__ __forceinline__ uint64_t* full(int b) const { return bar + b; }
  __device__ __forceinline__ uint64_t* empty(int b) const { return bar + NB + b; }
  __device__ __forceinline__ uint64_t* window_release() const { return bar + 2 * NB; }
  __device__ __forceinline__ uint64_t* window_full() const { return bar + 2 * NB + 1; }
  __device__ __forceinline__ unsigned char* window_mem(unsigned char* dsmem) const {
    return dsmem + bytes();
  }

  // Per-row operand q of row r for the epilogue.
  __device__ __forceinline__ V row(int q, int r) const {
    return rows_staged ? cur_rows[q * kRowStride + (r - row_base)] : rsrc[q][r];
  }

  __device__ __forceinline__ void setup(unsigned char* dsmem) {
    idx0 = reinterpret_cast<int*>(dsmem);
    val0 = reinterpret_cast<V*>(idx0 + NB * kStride);
    row0 = val0 + NB * kStride;
    ptr0 = reinterpret_cast<int*>(row0 + NB * NR * kRowStride);
    meta0 = ptr0 + NB * kRowStride;
    bar = reinterpret_cast<uint64_t*>(meta0 + NB * kMeta);
    cur_rows = nullptr;
    row_base = 0;
    rows_staged = false;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        mbar_init(full(b), 1);
        mbar_init(empty(b), kConsumerWarps);
      }
      mbar_init(window_release(), kConsumerWarps);
      mbar_init(window_full(), 1);
      fence_mbar_init();
    }
    __syncthreads();
  }

  // Producer: start the copies of a tile (entries; for a row tile also its row pointers and
  // its rows' operands) into buffer b, and record the tile and its window id there (generic
  // stores, published to the consumers by the arrival on the full barrier).
  __device__ __forceinline__ void issue(const TileSet<V>& ts, const Tile& tile, int win, int b) {
    int* m = meta(b);
    m[0] = tile.r0;
    m[1] = tile.r1;
    m[2] = tile.k0;
    m[3] = tile.k1;
    m[4] = win;
    const int a0 = tile.k0 & ~3;
    const int a1 = (tile.k1 + 3) & ~3;
    const uint32_t n = static_cast<uint32_t>(a1 - a0);
    const uint32_t bi = n * static_cast<uint32_t>(sizeof(int));
    const uint32_t bv = n * static_cast<uint32_t>(sizeof(V));
    uint32_t br = 0, bp = 0;
    int w0 = 0;
    if (tile.r1 >= 0) {
      w0 = tile.r0 & ~3;
      bp = static_cast<uint32_t>(((tile.r1 + 1 + 3) & ~3) - w0) * 4u;
      if (NR > 0) {
        br = static_cast<uint32_t>(((tile.r1 + 3) & ~3) - w0) * static_cast<uint32_t>(sizeof(V));
      }
    }
    const uint32_t total = bi + bv + bp + NR * br;
    if (total == 0) {
      mbar_arrive(full(b));
      return;
    }
    mbar_arrive_expect_tx(full(b), total);
    if (n > 0) {
      bulk_copy_g2s(idx(b), ts.idx + a0, bi, full(b));
      bulk_copy_g2s(val(b), ts.val + a0, bv, full(b));
    }
    if (bp > 0) bulk_copy_g2s(ptrs(b), ts.ptr + w0, bp, full(b));
    if (br > 0) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        bulk_copy_g2s(rows(b) + q * kRowStride, rsrc[q] + w0, br, full(b));
      }
    }
  }
};

// ---- Windows of the gathered vector ---------------------------------------------------------
// No staging: every gather reads global memory.
struct NoWindow {
  template <typename V, int NB, int NR, int CT>
  __device__ __forceinline__ bool sync(TilePipe<V, NB, NR, CT>&, const TileSet<V>&, int,
                                       volatile int*) {
    return true;
  }
};

// A staged slice [lo, lo + staged) of the vector `src` of element type G in shared memory.
// sync() runs in every consumer thread before a tile is worked on (the tile's window id is
// uniform, so the branch is too). When the id differs from the slice held, every consumer
// warp reports that it is done with the earlier tiles (window release barrier), consumer
// thread 0 then copies the new slice in, and all wait for it (window full barrier). get(i)
// reads element i from the slice when the tile has a window and i is in it, else from global
// memory.
template <typename G>
struct Window {
  const G* src;
  G* buf;
  int lo;       // staged slice start
  int staged;   // staged slice length
  int active;   // length usable for the current tile (0 when the tile has no window)
  int id;       // staged window id, -1 before the first
  uint32_t phase;
  bool pending;  // a copy was issued and not yet seen complete (consumer thread 0)

  template <typename V, int NB, int NR, int CT>
  __device__ __forceinline__ void setup(const G* vec, TilePipe<V, NB, NR, CT>& pipe,
                                        unsigned char* dsmem) {
    src = vec;
    buf = reinterpret_cast<G*>(pipe.window_mem(dsmem));
    lo = 0;
    staged = 0;
    active = 0;
    id = -1;
    phase = 0;
    pending = false;
  }

  template <typename V, int NB, int NR, int CT>
  __device__ __forceinline__ bool sync(TilePipe<V, NB, NR, CT>& pipe, const TileSet<V>& ts,
                                       int w, volatile int* abort_flag) {
    if (ts.wmax == 0 || w < 0) {
      active = 0;
      return true;
    }
    if (w != id) {
      const int2 r = __ldg(ts.windows + w);
      __syncwarp();
      if ((threadIdx.x & 31) == 0) mbar_arrive(pipe.window_release());
      if (threadIdx.x == 0) {
        if (mbar_wait_or_abort(pipe.window_release(), phase, abort_flag)) {
          const uint32_t bytes = static_cast<uint32_t>(r.y) * static_cast<uint32_t>(sizeof(G));
          fence_proxy_async_smem();
          mbar_arrive_expect_tx(pipe.window_full(), bytes);
          bulk_copy_g2s(buf, src + r.x, bytes, pipe.window_full());
          pending = true;
        } else {
          *abort_flag = 1;
        }
      }
      if (!mbar_wait_or_abort(pipe.window_full(), phase, abort_flag)) {
        *abort_flag = 1;
        return false;
      }
      pending = false;
      phase ^= 1u;
      id = w;
      lo = r.x;
      staged = r.y;
    }
    active = staged;
    return true;
  }

  // Consumer thread 0, after an abort: give a copy still in flight a bounded time to land.
  template <typename V, int NB, int NR, int CT>
  __device__ __forceinline__ void drain_copy(TilePipe<V, NB, NR, CT>& pipe) {
    if (pending) mbar_wait_bounded(pipe.window_full(), phase);
  }

  __device__ __forceinline__ G get(int i) const {
    const unsigned o = static_cast<unsigned>(i - lo);
    return o < static_cast<unsigned>(active) ? buf[o] : __ldg(src + i);
  }
};

template <typename V, int NB, int NR, int CT>
__device__ __forceinline__ void drain_window(NoWindow&, TilePipe<V, NB, NR, CT>&) {}
template <typename G, typename V, int NB, int NR, int CT>
__device__ __forceinline__ void drain_window(Window<G>& w, TilePipe<V, NB, NR, CT>& pipe) {
  w.drain_copy(pipe);
}

// Visit the tiles of this block (launched with CT + 32 threads). Per short tile,
// `lanes` consumer threads share row r and call
//   gather(col, value, acc) for each entry of the row (ascending), acc an A[NP],
//   epi(row, acc) once the row is summed (lane 0 of the row's group).
// A chunk tile is walked by one consumer warp, reduced in double across its lanes in a fixed
// order, and its lane 0 writes chunk_part[slot * NP + q]. `win` is synchronised before each
// tile (see Window). Returns false -- in every thread -- if a wait gave up; the copies still
// in flight are then given a bounded time to land before the caller records the error.
template <int NP, typename A, typename V, int NB, int NR, int CT, typename W, typename Gather,
          typename Epi>
__device__ __forceinline__ bool run_tiles(TilePipe<V, NB, NR, CT>& pipe, const TileSet<V>& ts,
                                          W& win,
                                          double* chunk_part, Gather gather, Epi epi) {
  __shared__ volatile int s_abort;
  __shared__ int s_issued;
  if (threadIdx.x == 0) {
    s_abort = 0;
    s_issued = 0;
  }
  __syncthreads();
  int first, last;
  block_tile_range(ts.ntiles, first, last);
  const int count = last - first;
  const int lane = static_cast<int>(threadIdx.x) & 31;
  if (threadIdx.x >= CT) {
    // Producer warp, lane 0. Each tile record is read one tile early, so the global load
    // overlaps the wait for a free buffer.
    if (lane == 0 && count > 0) {
      Tile rec = ts.tiles[first];
      int rec_win = ts.wmax > 0 ? __ldg(ts.tile_win + first) : -1;
      int j = 0;
      for (; j < count; ++j) {
        const int b = j % NB;
        if (j >= NB && !mbar_wait_or_abort(pipe.empty(b),
                                           static_cast<uint32_t>(((j / NB) - 1) & 1), &s_abort)) {
          s_abort = 1;
          break;
        }
        fence_proxy_async_smem();
        pipe.issue(ts, rec, rec_win, b);
        if (j + 1 < count) {
          rec = ts.tiles[first + j + 1];
          rec_win = ts.wmax > 0 ? __ldg(ts.tile_win + first + j + 1) : -1;
        }
      }
      s_issued = j;
    }
  } else {
    const int warp = static_cast<int>(threadIdx.x) >> 5;
    for (int i = 0; i < count; ++i) {
      const int b = i % NB;
      if (!mbar_wait_or_abort(pipe.full(b), static_cast<uint32_t>((i / NB) & 1), &s_abort)) {
        s_abort = 1;
        break;
      }
      const int* m = pipe.meta(b);
      const Tile tile{m[0], m[1], m[2], m[3]};
      if (!win.sync(pipe, ts, m[4], &s_abort)) break;
      const int base = tile.k0 & ~3;
      const int* __restrict__ sidx = pipe.idx(b);
      const V* __restrict__ sval = pipe.val(b);
      if (tile.r1 == tile.r0 + 1 && tile.k1 - tile.k0 > kWarpRowMin) {
        // A warp row: lanes take entries l, l + 32, ... in order, a fixed xor tree adds them,
        // and lane 0 runs the epilogue with the row's staged operands.
        if (warp == i % (CT / 32)) {
          if (NR > 0) {
            pipe.cur_rows = pipe.rows(b);
            pipe.row_base = tile.r0 & ~3;
            pipe.rows_staged = true;
          }
          A acc[NP];
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[q] = A(0);
          for (int k = tile.k0 - base + lane; k < tile.k1 - base; k += 32) {
            gather(sidx[k], sval[k], acc);
          }
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[q] = warp_sum(acc[q]);
          if (lane == 0) epi(tile.r0, acc);
        }
      } else if (tile.r1 < 0) {
        if (warp == i % (CT / 32)) {
          A acc[NP];
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[q] = A(0);
          for (int k = tile.k0 - base + lane; k < tile.k1 - base; k += 32) {
            gather(sidx[k], sval[k], acc);
          }
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const double d = warp_sum(static_cast<double>(acc[q]));
            if (lane == 0) chunk_part[(-tile.r1 - 1) * NP + q] = d;
          }
        }
      } else {
        // `lanes` consecutive threads share row r: lane l sums entries l, l + lanes, ... in
        // ascending order, then a fixed xor tree adds the lanes' sums (lanes are aligned
        // groups inside a warp, and every thread takes part in the shuffles).
        const int pbase = tile.r0 & ~3;
        if (NR > 0) {
          pipe.cur_rows = pipe.rows(b);
          pipe.row_base = pbase;
          pipe.rows_staged = true;
        }
        const int* sptr = pipe.ptrs(b);
        const int lanes = ts.lanes;
        const int sub = static_cast<int>(threadIdx.x) & (lanes - 1);
        const int r = tile.r0 + static_cast<int>(threadIdx.x) / lanes;
        A acc[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] = A(0);
        if (r < tile.r1) {
          const int a = sptr[r - pbase] - base, e = sptr[r + 1 - pbase] - base;
#pragma unroll 4
          for (int k = a + sub; k < e; k += lanes) gather(sidx[k], sval[k], acc);
        }
        for (int o = lanes >> 1; o > 0; o >>= 1) {
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
        }
        if (r < tile.r1 && sub == 0) epi(r, acc);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(pipe.empty(b));
    }
  }
  pipe.rows_staged = false;
  __syncthreads();
  if (!s_abort) return true;
  // Abort: the producer waits (bounded) for the copies it issued into the buffers, and
  // consumer thread 0 for a window copy, before the block may exit.
  if (threadIdx.x == CT) {
    const int issued = s_issued;
    for (int j = issued - NB > 0 ? issued - NB : 0; j < issued; ++j) {
      mbar_wait_bounded(pipe.full(j % NB), static_cast<uint32_t>((j / NB) & 1));
    }
  }
  if (threadIdx.x == 0) drain_window(win, pipe);
  __syncthreads();
  return false;
}

// The same without staging.
template <int NP, typename A, typename V, int NB, int NR, int CT, typename Gather,
          typename Epi>
__device__ __forceinline__ bool run_tiles(TilePipe<V, NB, NR, CT>& pipe, const TileSet<V>& ts,
                                          double* chunk_part, Gather gather, Epi epi) {
  NoWindow none;
  return run_tiles<NP, A>(pipe, ts, none, chunk_part, gather, epi);
}

// Last block only: the long rows, each combined from its chunk partials in chunk order (in
// double), then handed to the epilogue in the accumulator type A.
template <int NP, typename A = double, typename V, typename Epi>
__device__ __forceinline__ void run_long_rows(const TileSet<V>& ts, const double* chunk_part,
                                              Epi epi) {
  for (int l = threadIdx.x; l < ts.nlong; l += blockDim.x) {
    const LongRow lr = ts.longs[l];
    double acc[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) acc[q] = 0.0;
    for (int c = 0; c < lr.nchunks; ++c) {
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += __ldcg(chunk_part + (lr.chunk0 + c) * NP + q);
    }
    A out[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) out[q] = static_cast<A>(acc[q]);
    epi(lr.row, out);
  }
}

// Publish this block's NV partials; returns true in the last block to arrive (all threads).
template <int NV>
__device__ __forceinline__ bool arrive_last(double (&v)[NV], double* scratch, double* part,
                                            unsigned int* ticket) {
  double out[NV];
  block_sum<NV>(v, scratch, out);
  __shared__ int s_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) part[blockIdx.x * NV + q] = out[q];
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  const bool last = s_last != 0;
  if (last) __threadfence();
  return last;
}

// Last block: fixed-order sum of every block's partials, plus `extra` (already reduced).
template <int NV>
__device__ __forceinline__ void sum_partials(const double* part, int nblocks, double* scratch,
                                             double (&out)[NV]) {
  double a[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) a[q] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NV; ++q) a[q] += __ldcg(part + b * NV + q);
  }
  block_sum<NV>(a, scratch, out);
}

}  // namespace sgb

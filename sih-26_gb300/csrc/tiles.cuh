// tiles.cuh -- TMA-staged row tiles: the sparse-product engine under every pass.
//
// A TILE is a run of consecutive rows (of the CSR copy, or columns of the CSC copy) whose
// nonzeros fit one shared-memory buffer (kCap entries). A row longer than kCap is cut into
// CHUNK tiles of at most kCap entries. Tiles are dealt to the blocks round-robin
// (tile t -> block t mod grid), so every sum below is taken in a fixed order and a run is
// bit-reproducible.
//
// Each block runs a two-stage pipeline over its tiles: thread 0 issues one bulk async copy
// (cp.async.bulk, the TMA engine's 1-D form) of the next tile's index and value ranges into
// the idle buffer, completing on an mbarrier, while all threads work on the current tile.
// Working on a tile: thread r walks row r of the tile in ascending index order, reading
// (index, value) from shared memory and gathering the vector entries from global memory
// (L2-resident for the vector sizes here), and accumulates with FMA. A chunk tile is walked
// by all threads and reduced across the block into a per-chunk partial; the chunks of a long
// row are combined in chunk order by the last block of the kernel.
//
// Copies must start on 16 bytes and move a multiple of 16 bytes, so a tile's range is
// widened to multiples of 4 entries on both sides; the device arrays carry kPad entries of
// padding so the widened range never leaves the allocation. Every mbarrier wait is bounded:
// a wait that gives up records an error in the control block and the kernel returns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace sgb {

constexpr int kCap = 2048;        // entries per tile buffer
constexpr int kSlack = 8;         // widening of a tile range to 16-byte boundaries
constexpr int kPad = 8;           // padding entries at the end of every index / value array
constexpr int kTileThreads = 256; // threads per tile block (max rows per tile)
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
                        // holds at most kTileThreads / lanes rows
};

// Lanes per row for a pattern with `avg` entries per row: the smallest power of two for
// which kTileThreads / lanes rows of average length fill one buffer, so that every thread
// of the block has entries to sum.
inline int choose_lanes(double avg) {
  int lanes = 1;
  while (lanes < 32 && (static_cast<double>(kTileThreads) / lanes) * avg > kCap) lanes *= 2;
  return lanes;
}

// Bytes of dynamic shared memory a tile kernel over value type V needs.
template <typename V>
constexpr int tile_smem_bytes() {
  return 2 * (kCap + kSlack) * static_cast<int>(sizeof(int) + sizeof(V)) + 64;
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

// ---- The pipeline --------------------------------------------------------------------------
template <typename V>
struct TilePipe {
  // Buffer b's entries start at idx0 + b * kStride / val0 + b * kStride (computed, never an
  // array indexed by b, so the pointers stay in registers).
  static constexpr int kStride = kCap + kSlack;
  int* idx0;
  V* val0;
  uint64_t* bar;

  __device__ __forceinline__ int* idx(int b) const { return idx0 + b * kStride; }
  __device__ __forceinline__ V* val(int b) const { return val0 + b * kStride; }

  __device__ __forceinline__ void setup(unsigned char* dsmem) {
    idx0 = reinterpret_cast<int*>(dsmem);
    val0 = reinterpret_cast<V*>(idx0 + 2 * kStride);
    bar = reinterpret_cast<uint64_t*>(val0 + 2 * kStride);
    if (threadIdx.x == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      fence_mbar_init();
    }
    __syncthreads();
  }

  // Thread 0: start the copy of tile t into buffer b.
  __device__ __forceinline__ void issue(const TileSet<V>& ts, int t, int b) {
    const Tile tile = ts.tiles[t];
    const int a0 = tile.k0 & ~3;
    const int a1 = (tile.k1 + 3) & ~3;
    const uint32_t n = static_cast<uint32_t>(a1 - a0);
    if (n == 0) {
      mbar_arrive(&bar[b]);
      return;
    }
    const uint32_t bi = n * static_cast<uint32_t>(sizeof(int));
    const uint32_t bv = n * static_cast<uint32_t>(sizeof(V));
    mbar_arrive_expect_tx(&bar[b], bi + bv);
    bulk_copy_g2s(idx(b), ts.idx + a0, bi, &bar[b]);
    bulk_copy_g2s(val(b), ts.val + a0, bv, &bar[b]);
  }
};

// Visit the tiles of this block. Per short tile, thread r calls
//   gather(col, value, acc) for each entry of row r0 + r (ascending), acc an A[NP],
//   epi(row, acc) once the row is summed.
// Per chunk tile, the entries are spread over the block, reduced in double, and thread 0
// writes chunk_part[slot * NP + q]. Returns false if a copy did not complete in time (the
// caller records the error; every thread returns the same value).
template <int NP, typename A, typename V, typename Gather, typename Epi>
__device__ __forceinline__ bool run_tiles(TilePipe<V>& pipe, const TileSet<V>& ts,
                                          double* chunk_part, double* scratch, Gather gather,
                                          Epi epi) {
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  const int G = gridDim.x;
  int it = 0;
  if (threadIdx.x == 0 && static_cast<int>(blockIdx.x) < ts.ntiles) pipe.issue(ts, blockIdx.x, 0);
  __syncthreads();
  for (int t = blockIdx.x; t < ts.ntiles; t += G, ++it) {
    const int b = it & 1;
    const int tn = t + G;
    if (threadIdx.x == 0) {
      if (tn < ts.ntiles) {
        fence_proxy_async_smem();
        pipe.issue(ts, tn, b ^ 1);
      }
      long long spins = 0;
      while (!mbar_try_wait(&pipe.bar[b], static_cast<uint32_t>((it >> 1) & 1))) {
        if (++spins > kWaitLimit) {
          s_abort = 1;
          break;
        }
      }
    }
    __syncthreads();
    if (s_abort) return false;
    const Tile tile = ts.tiles[t];
    const int base = tile.k0 & ~3;
    const int* __restrict__ sidx = pipe.idx(b);
    const V* __restrict__ sval = pipe.val(b);
    if (tile.r1 < 0) {
      A acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = A(0);
      for (int k = tile.k0 - base + threadIdx.x; k < tile.k1 - base; k += blockDim.x) {
        gather(sidx[k], sval[k], acc);
      }
      double d[NP], out[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) d[q] = static_cast<double>(acc[q]);
      block_sum<NP>(d, scratch, out);
      if (threadIdx.x == 0) {
        const int slot = -tile.r1 - 1;
#pragma unroll
        for (int q = 0; q < NP; ++q) chunk_part[slot * NP + q] = out[q];
      }
    } else {
      // `lanes` consecutive threads share row r: lane l sums entries l, l + lanes, ... in
      // ascending order, then a fixed xor tree adds the lanes' sums (lanes are aligned
      // groups inside a warp, and every thread takes part in the shuffles).
      const int lanes = ts.lanes;
      const int lane = static_cast<int>(threadIdx.x) & (lanes - 1);
      const int r = tile.r0 + static_cast<int>(threadIdx.x) / lanes;
      A acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = A(0);
      if (r < tile.r1) {
        const int a = ts.ptr[r] - base, e = ts.ptr[r + 1] - base;
#pragma unroll 4
        for (int k = a + lane; k < e; k += lanes) gather(sidx[k], sval[k], acc);
      }
      for (int o = lanes >> 1; o > 0; o >>= 1) {
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
      }
      if (r < tile.r1 && lane == 0) epi(r, acc);
    }
    __syncthreads();
  }
  return true;
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

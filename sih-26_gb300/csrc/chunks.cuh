// chunks.cuh -- warp chunks: the sparse-product engine of the PDHG step passes.
//
// A CHUNK is a run of at most kChunkRows consecutive rows (of the CSR copy, or columns of the
// CSC copy) holding at most CH nonzeros; a row longer than CH is cut into PIECES of CH
// entries. Each warp of a block works through its own chunks, one at a time, with no
// barrier between warps:
//   1. its lanes load the chunk's indices and values straight from global memory, lane l
//      taking entries l, l + 32, ... (every load coalesced, streamed past L1), and the
//      per-row operands of the epilogue, lane l taking row r0 + l;
//   2. they gather the vector entry of each nonzero -- from the block's staged WINDOW of the
//      vector in shared memory, or from L2 when the window does not hold it -- and stage the
//      (value, gathered) pairs in the warp's shared buffer;
//   3. `L` lanes per row (the largest power of two with 32 / L >= rows) sum each row from
//      the buffer with FMA, in a fixed order (lane s takes entries s, s + L, ...; then a fixed
//      xor tree), and the row's first lane runs the epilogue with the operands shuffled to
//      it. A piece of a long row is summed by the whole warp into a piece partial; the last
//      block of the kernel combines the pieces of each long row in order.
// The stream loads of every warp in flight at once are what keep HBM busy: registers hold
// them, so shared memory is left to the window.
//
// WINDOWS. Random 4- or 8-byte gathers from L2 cost one 32-byte sector request each, and an
// SM retires about one sector request per clock: far below what the streamed matrix needs.
// So a block keeps a slice [lo, lo + len) of the gathered vector in shared memory, copied in
// by one bulk copy (cp.async.bulk) whenever its chunks move to another slice. A block owns
// a contiguous run of chunks; chunks that share a slice form a SEGMENT; the block stages each
// segment's slice in turn. Blocks are cut by a cost model (entries, plus a fixed cost per
// slice staged) so that a block that must stage two slices takes fewer entries.
//
// SPLIT LAYOUTS. A gather that misses the window stalls its whole warp on L2 latency, and in
// a chunk of 256 entries almost every warp-wide gather has a lane that misses when even 8% of
// the entries fall outside. So where a window covers most but not all of a layout's entries,
// the layout is split: the entries inside each row's window form the main matrix (gathered
// from shared memory only), the rest an OUTER matrix of their own. Each block first sums the
// outer entries of its own rows (plain L2 gathers, while its first window copy is in flight)
// into outer[row], and the main loop adds outer[row] to each row's sum before its epilogue.
//
// Every wait is bounded: a wait that gives up raises the block's abort flag, the remaining
// chunks are skipped, the copy still in flight is given a bounded time to land, and the
// caller records the error.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "tiles.cuh"

namespace sgb {

constexpr int kChunkRows = 31;     // rows per chunk (lane 31 reads the closing row pointer)
constexpr int kChunkCapF = 256;    // entries per chunk, FP32 layouts
constexpr int kChunkThreads = 1024;
// The largest window a chunk kernel stages. Shared memory and L1 share each SM's 256 KB, and
// the step passes' per-row operand and row-pointer loads go through L1: on the 1M x 2M
// block-angular LP the FP32 column pass ran in 61 us with a 128 KB window and in 84 us with
// the 160 KB that fits beside the warp buffers (the row pass: 89 us against 104 us).
constexpr int kWindowBytesMax = 128 * 1024;

// Consecutive chunks of one block that gather from the same staged slice [lo, lo + len) of
// the vector (len = 0: no slice, every gather from global memory).
struct ChunkSeg {
  int c0, c1;
  int lo, len;
};

// A chunk record is a Tile: rows [r0, r1), entries [k0, k1); r1 < 0 marks a piece of a long
// row whose partial goes to piece slot -r1 - 1.
template <typename T>
struct ChunkSet {
  const int* ptr;        // rows + 1 (main part)
  const int* idx;        // nnz (+ kPad)
  const T* val;          // nnz (+ kPad)
  const Tile* chunks;
  const ChunkSeg* segs;
  const int* seg_start;  // per block: its segments [seg_start[b], seg_start[b + 1])
  const LongRow* longs;  // long rows and their piece slots
  int nlong;
  int npieces;
  int nrows;
  int wmax;              // window capacity in gathered elements (0: the layout stages none)
  // Split layouts: the out-of-window entries as a CSR of their own. Block b sums the outer
  // entries of its rows in ROUNDS (row ranges orounds[oround_start[b] .. oround_start[b + 1]),
  // each with at most as many outer entries as the block's warp buffers hold); outer holds
  // NP sums per row.
  const int* optr;
  const int* oidx;
  const T* oval;
  const int2* orounds;
  const int* oround_start;
  T* outer;              // nullptr: not split
};

// ---- PTX helpers ---------------------------------------------------------------------------
__device__ __forceinline__ int ld_stream(const int* p) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// Components of a gathered element.
template <typename T>
__device__ __forceinline__ void split_gathered(float g, T (&c)[1]) { c[0] = g; }
template <typename T>
__device__ __forceinline__ void split_gathered(double g, T (&c)[1]) { c[0] = g; }
template <typename T>
__device__ __forceinline__ void split_gathered(double2 g, T (&c)[2]) {
  c[0] = g.x;
  c[1] = g.y;
}

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <>
__device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }

// Whether a layout's warps stage products (one FP32 multiply per entry, summed with adds) or
// (value, gathered) pairs (summed with one FMA per entry and product). FP32 stages products:
// half the shared-memory traffic. FP64 stages pairs: GB300 retires FP64 at a few operations
// per clock per SM, so a multiply and an add per entry would cost twice the FMA.
template <typename T>
struct StageProducts {
  static constexpr bool value = sizeof(T) == sizeof(float);
};

// Dynamic shared memory of a chunk kernel: per-warp buffers, the window barrier, the window.
template <typename T, typename G, int NP, int CH>
struct ChunkSmem {
  static constexpr int kBufBytes =
      CH * (StageProducts<T>::value ? NP : 1 + NP) * static_cast<int>(sizeof(T));
  __host__ __device__ static constexpr int bytes(int warps, int wmax) {
    return warps * kBufBytes + 128 + ((wmax * static_cast<int>(sizeof(G)) + 127) & ~127);
  }
};

// Lanes per row for a chunk of R rows: the largest power of two L with 32 / L >= R.
__device__ __forceinline__ int chunk_lanes(int R) {
  const int p = R <= 1 ? 0 : 32 - __clz(R - 1);  // the smallest p with 2^p >= R
  return 32 >> p;
}

// One chunk: stream, gather, stage, sum, epilogue (all lanes of the warp call it).
//   gather(col) -> G          the vector element of column col
//   load(row, ops)            the row's NR epilogue operands (lane-per-row, at chunk start)
//   epi(row, sums, ops)       once per row, on the row's first lane
template <int NP, int NR, typename T, typename G, int CH, bool OUTER, typename Gather,
          typename Load, typename Epi>
__device__ __forceinline__ void chunk_step(const int* __restrict__ ptr, const int* __restrict__ idx,
                                           const T* __restrict__ val, const Tile& ch, T* buf,
                                           const T* __restrict__ outer, double* piece_part,
                                           Gather gather, Load load, Epi epi) {
  constexpr int J = CH / 32;
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const bool piece = ch.r1 < 0;
  const int R = piece ? 0 : ch.r1 - ch.r0;
  const int n = ch.k1 - ch.k0;
  int col[J];
  T a[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = ch.k0 + lane + 32 * j;
    const bool in = lane + 32 * j < n;
    col[j] = in ? ld_stream(idx + k) : -1;
    a[j] = in ? ld_stream(val + k) : T(0);
  }
  int pr = 0;
  T ops[NR > 0 ? NR : 1];
  T out[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) out[q] = T(0);
  if (!piece) {
    if (lane <= R) pr = __ldg(ptr + ch.r0 + lane);
    if (lane < R) {
      load(ch.r0 + lane, ops);
      if (OUTER) {
#pragma unroll
        for (int q = 0; q < NP; ++q) out[q] = outer[(ch.r0 + lane) * NP + q];
      }
    }
  }
  constexpr bool kProducts = StageProducts<T>::value;
  // Pairs: bv holds the values, bg the NP gathered components; products: bg the NP products.
  T* bv = buf;
  T* bg = kProducts ? buf : buf + CH;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    T c[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) c[q] = T(0);
    if (col[j] >= 0) split_gathered(gather(col[j]), c);
    // Past the chunk's end the entry is a zero that no row reads.
    if (kProducts) {
#pragma unroll
      for (int q = 0; q < NP; ++q) bg[q * CH + lane + 32 * j] = a[j] * c[q];
    } else {
      bv[lane + 32 * j] = a[j];
#pragma unroll
      for (int q = 0; q < NP; ++q) bg[q * CH + lane + 32 * j] = c[q];
    }
  }
  __syncwarp();
  // The sum of entry k's term q in order: an add of the staged product, or an FMA of the
  // staged pair.
  auto term = [&](int q, int k, T acc) {
    return kProducts ? acc + bg[q * CH + k] : fma_t(bv[k], bg[q * CH + k], acc);
  };
  if (piece) {
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      T s = T(0);
      for (int k = lane; k < n; k += 32) s = term(q, k, s);
      const double d = warp_sum(static_cast<double>(s));
      if (lane == 0) piece_part[(-ch.r1 - 1) * NP + q] = d;
    }
  } else {
    const int L = chunk_lanes(R);
    const int g = lane / L, sub = lane & (L - 1);
    const int ra = __shfl_sync(0xffffffffu, pr, g & 31) - ch.k0;
    const int re = __shfl_sync(0xffffffffu, pr, (g + 1) & 31) - ch.k0;
    T s[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) s[q] = T(0);
    if (g < R) {
      for (int k = ra + sub; k < re; k += L) {
#pragma unroll
        for (int q = 0; q < NP; ++q) s[q] = term(q, k, s[q]);
      }
    }
    for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < NP; ++q) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    }
    T og[NR > 0 ? NR : 1];
#pragma unroll
    for (int q = 0; q < NR; ++q) og[q] = __shfl_sync(0xffffffffu, ops[q], g & 31);
    if (OUTER) {
#pragma unroll
      for (int q = 0; q < NP; ++q) s[q] += __shfl_sync(0xffffffffu, out[q], g & 31);
    }
    if (g < R && sub == 0) epi(ch.r0 + g, s, og);
  }
  __syncwarp();
}

// The outer sums of a split layout's rows, for this block: in each round, every thread takes
// outer entries e, e + blockDim, ... of the round's contiguous entry range (coalesced loads,
// gathers from global memory) and stages their products (or pairs) in the warp buffers, then
// every thread sums the rows r, r + blockDim, ... of the round in entry order into outer[r].
// All threads call it; it ends with the block synchronised.
template <int NP, typename T, typename G>
__device__ __forceinline__ void outer_sums(const ChunkSet<T>& cs, const G* __restrict__ vec,
                                           T* stage) {
  constexpr bool kProducts = StageProducts<T>::value;
  const int B = static_cast<int>(blockDim.x);
  const int t = static_cast<int>(threadIdx.x);
  for (int q0 = cs.oround_start[blockIdx.x]; q0 < cs.oround_start[blockIdx.x + 1]; ++q0) {
    const int2 rr = cs.orounds[q0];
    const int e0 = __ldg(cs.optr + rr.x), e1 = __ldg(cs.optr + rr.y);
    const int count = e1 - e0;
    // Stage: pairs put the value at [k] and component q at [(1 + q) * count + k]. A thread
    // takes kOuterBatch entries at a time and issues all their index and value loads, then
    // all their gathers, so it waits for two latencies per batch, not two per entry.
    constexpr int kOuterBatch = 8;
    for (int k0 = t; k0 < count; k0 += B * kOuterBatch) {
      int ix[kOuterBatch];
      T av[kOuterBatch];
#pragma unroll
      for (int u = 0; u < kOuterBatch; ++u) {
        const int k = k0 + u * B;
        ix[u] = k < count ? ld_stream(cs.oidx + e0 + k) : -1;
        av[u] = k < count ? ld_stream(cs.oval + e0 + k) : T(0);
      }
      G g[kOuterBatch];
#pragma unroll
      for (int u = 0; u < kOuterBatch; ++u) g[u] = ix[u] >= 0 ? __ldg(vec + ix[u]) : G{};
#pragma unroll
      for (int u = 0; u < kOuterBatch; ++u) {
        const int k = k0 + u * B;
        if (k >= count) break;
        T c[NP];
        split_gathered(g[u], c);
        if (kProducts) {
#pragma unroll
          for (int q = 0; q < NP; ++q) stage[q * count + k] = av[u] * c[q];
        } else {
          stage[k] = av[u];
#pragma unroll
          for (int q = 0; q < NP; ++q) stage[(1 + q) * count + k] = c[q];
        }
      }
    }
    __syncthreads();
    for (int r = rr.x + t; r < rr.y; r += B) {
      const int a0 = __ldg(cs.optr + r) - e0, a1 = __ldg(cs.optr + r + 1) - e0;
      T s[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) s[q] = T(0);
      for (int k = a0; k < a1; ++k) {
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          s[q] = kProducts ? s[q] + stage[q * count + k]
                           : fma_t(stage[k], stage[(1 + q) * count + k], s[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) cs.outer[r * NP + q] = s[q];
    }
    __syncthreads();
  }
}

template <bool OUTER, int NP, int NR, typename T, typename G, int CH, typename Load, typename Epi>
__device__ __forceinline__ bool run_chunks_impl(const ChunkSet<T>& cs, const G* __restrict__ vec,
                                                unsigned char* dsmem, double* piece_part,
                                                Load load, Epi epi) {
  __shared__ volatile int s_abort;
  const int W = static_cast<int>(blockDim.x) >> 5;
  const int warp = static_cast<int>(threadIdx.x) >> 5;
  T* buf = reinterpret_cast<T*>(dsmem + warp * ChunkSmem<T, G, NP, CH>::kBufBytes);
  uint64_t* winbar =
      reinterpret_cast<uint64_t*>(dsmem + W * ChunkSmem<T, G, NP, CH>::kBufBytes);
  G* win = reinterpret_cast<G*>(dsmem + W * ChunkSmem<T, G, NP, CH>::kBufBytes + 128);
  if (threadIdx.x == 0) {
    s_abort = 0;
    mbar_init(winbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int s0 = cs.seg_start[blockIdx.x], s1 = cs.seg_start[blockIdx.x + 1];
  uint32_t phase = 0;
  bool pending = false;  // thread 0: a window copy issued and not yet seen complete

  // The first window copy is issued at once; a split layout sums its outer entries while it
  // is in flight.
  if (s0 < s1 && cs.segs[s0].len > 0 && threadIdx.x == 0) {
    const ChunkSeg sg = cs.segs[s0];
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(winbar, static_cast<uint32_t>(sg.len) * sizeof(G));
    bulk_copy_g2s(win, vec + sg.lo, static_cast<uint32_t>(sg.len) * sizeof(G), winbar);
    pending = true;
  }
  if (OUTER) outer_sums<NP>(cs, vec, reinterpret_cast<T*>(dsmem));

  for (int s = s0; s < s1; ++s) {
    const ChunkSeg sg = cs.segs[s];
    if (sg.len > 0) {
      if (s != s0) {
        __syncthreads();  // every warp is done with the slice held
        if (!s_abort && threadIdx.x == 0) {
          fence_proxy_async_smem();
          mbar_arrive_expect_tx(winbar, static_cast<uint32_t>(sg.len) * sizeof(G));
          bulk_copy_g2s(win, vec + sg.lo, static_cast<uint32_t>(sg.len) * sizeof(G), winbar);
          pending = true;
        }
      }
      if (!s_abort) {
        if (mbar_wait_or_abort(winbar, phase, &s_abort)) {
          if (threadIdx.x == 0) pending = false;
        } else {
          s_abort = 1;
        }
      }
      phase ^= 1u;
    }
    const int lo = sg.lo, len = sg.len;
    auto gather = [&](int c) {
      const unsigned o = static_cast<unsigned>(c - lo);
      return o < static_cast<unsigned>(len) ? win[o] : __ldg(vec + c);
    };
    // The next chunk's record is loaded while this one is worked on: the stream loads of a
    // chunk wait for its record.
    Tile next = sg.c0 + warp < sg.c1 ? cs.chunks[sg.c0 + warp] : Tile{0, 0, 0, 0};
    for (int c = sg.c0 + warp; c < sg.c1; c += W) {
      if (s_abort) break;
      const Tile ch = next;
      if (c + W < sg.c1) next = cs.chunks[c + W];
      chunk_step<NP, NR, T, G, CH, OUTER>(cs.ptr, cs.idx, cs.val, ch, buf, cs.outer, piece_part,
                                          gather, load, epi);
    }
  }
  __syncthreads();
  if (!s_abort) return true;
  // A window copy still in flight must land before the block exits (bounded).
  if (threadIdx.x == 0 && pending) mbar_wait_bounded(winbar, phase ^ 1u);
  __syncthreads();
  return false;
}

// Visit this block's chunks (kernel launched with a multiple of 32 threads, every thread
// calls it). Returns false -- in every thread -- if a wait gave up.
template <int NP, int NR, typename T, typename G, int CH, typename Load, typename Epi>
__device__ __forceinline__ bool run_chunks(const ChunkSet<T>& cs, const G* __restrict__ vec,
                                           unsigned char* dsmem, double* piece_part, Load load,
                                           Epi epi) {
  return cs.outer != nullptr
             ? run_chunks_impl<true, NP, NR, T, G, CH>(cs, vec, dsmem, piece_part, load, epi)
             : run_chunks_impl<false, NP, NR, T, G, CH>(cs, vec, dsmem, piece_part, load, epi);
}

// Last block only: each long row combined from its piece partials in piece order (double),
// then handed to the epilogue with its operands.
template <int NP, int NR, typename T, typename Load, typename Epi>
__device__ __forceinline__ void run_chunk_long_rows(const ChunkSet<T>& cs,
                                                    const double* piece_part, Load load,
                                                    Epi epi) {
  for (int l = threadIdx.x; l < cs.nlong; l += blockDim.x) {
    const LongRow lr = cs.longs[l];
    double acc[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) acc[q] = 0.0;
    for (int c = 0; c < lr.nchunks; ++c) {
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += __ldcg(piece_part + (lr.chunk0 + c) * NP + q);
    }
    T s[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) s[q] = static_cast<T>(acc[q]);
    T ops[NR > 0 ? NR : 1];
    load(lr.row, ops);
    epi(lr.row, s, ops);
  }
}

}  // namespace sgb

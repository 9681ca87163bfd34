// layout_check.cu -- host-only checks of the tile and window layouts the kernels rely on.
//
// Built by tests/test_host_layout.py against the engine's objects and run on the CPU (no
// CUDA call is made). For random and banded sparsity patterns, every lane count and both
// block sizes, it checks that:
//   * the tiles cover the lines in order, short tiles within min(kMaxTileRows, threads /
//     lanes) rows and kCap entries, rows longer than kCap as consecutive chunk tiles;
//   * every bulk copy a tile issues (entries widened to 4-element bounds, row pointers, the
//     rows' operand slices) fits its shared-memory buffer and stays inside the padded arrays;
//   * every window starts and ends on a 4-element bound, holds at most wmax elements, lies
//     inside the padded gathered vector, and the staged count build_windows returns is the
//     number of entries that fall inside their tile's window;
//   * with one lane per row, a row of more than kWarpRowMin entries has a tile of its own;
//   * the chunk plans of the FP32 step passes (plan_chunks): chunks cover the lines in order
//     within kChunkRows rows and `cap` entries, long rows as pieces; every block's segments
//     cover its chunks in order with windows on 4-element bounds inside the padded vector;
//     a split layout's main and outer parts partition the entries, every main entry of a
//     windowed chunk lies in its window, and the outer rounds write every row exactly once,
//     by the block whose chunks hold it, within the staging space;
// plus the FP32 lane rule and the step graph's launch count. Given a file, it checks the
// layouts the engine builds for that pattern instead (read_pattern).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "chunks.cuh"
#include "engine.hpp"
#include "kernels.cuh"
#include "tiles.cuh"

using namespace sgb;

namespace {

int g_failures = 0;

void fail(const char* what, long long a, long long b) {
  if (g_failures < 20) std::printf("FAIL: %s (%lld, %lld)\n", what, a, b);
  ++g_failures;
}

struct Pattern {
  int lines = 0;
  int extent = 0;
  std::vector<int> ptr;
  std::vector<int> idx;
};

// Row lengths: mostly short, some empty, a few around and far beyond kCap.
Pattern make_pattern(unsigned seed, int lines, int extent, bool banded) {
  std::mt19937 rng(seed);
  Pattern p;
  p.lines = lines;
  p.extent = extent;
  p.ptr.push_back(0);
  for (int r = 0; r < lines; ++r) {
    int len;
    const unsigned kind = rng() % 1000;
    if (kind < 20) {
      len = 0;
    } else if (kind < 23) {
      const int specials[] = {kCap, kCap + 1, 3 * kCap + 17};
      len = specials[rng() % 3];
    } else {
      len = 1 + static_cast<int>(rng() % 40);
    }
    for (int k = 0; k < len; ++k) {
      int c;
      if (banded) {
        const long long centre = static_cast<long long>(r) * extent / lines;
        const int spread = 600;
        c = static_cast<int>((centre + static_cast<int>(rng() % (2 * spread)) - spread +
                              extent) % extent);
        if (rng() % 10 == 0) c = static_cast<int>(rng() % extent);  // a far link
      } else {
        c = static_cast<int>(rng() % extent);
      }
      p.idx.push_back(c);
    }
    p.ptr.push_back(static_cast<int>(p.idx.size()));
  }
  return p;
}

void check_tiles(const Pattern& p, int lanes, int threads, const std::vector<Tile>& tiles,
                 const std::vector<LongRow>& longs, int nchunks) {
  const int max_rows = std::min(kMaxTileRows, threads / lanes);
  const long long nnz = p.ptr[p.lines];
  int row = 0;
  int chunk = 0;
  size_t li = 0;
  for (size_t t = 0; t < tiles.size(); ++t) {
    const Tile& tile = tiles[t];
    if (tile.k1 - tile.k0 > kCap) fail("tile entries > kCap", tile.k0, tile.k1);
    if (tile.k0 < 0 || tile.k1 > nnz || tile.k0 > tile.k1) fail("tile entry range", tile.k0, tile.k1);
    // The entry copy: widened to 4-element bounds, within the buffer and the padded arrays.
    const int a0 = tile.k0 & ~3, a1 = (tile.k1 + 3) & ~3;
    if (a1 - a0 > kCap + kSlack) fail("entry copy exceeds the buffer", a0, a1);
    if (a1 > nnz + kPad) fail("entry copy beyond the padded arrays", a1, nnz);
    if (tile.r1 < 0) {
      // A chunk tile of the long row `row`.
      if (li >= longs.size() || longs[li].row != tile.r0) fail("chunk tile without its long row", tile.r0, static_cast<long long>(li));
      if (-tile.r1 - 1 != chunk) fail("chunk slot order", -tile.r1 - 1, chunk);
      if (tile.r0 != row) fail("chunk tile row", tile.r0, row);
      const bool last = tile.k1 == p.ptr[row + 1];
      ++chunk;
      if (last) {
        if (li < longs.size() && longs[li].chunk0 + longs[li].nchunks != chunk) {
          fail("long row chunk count", longs[li].nchunks, chunk);
        }
        ++li;
        ++row;
      }
      continue;
    }
    if (tile.r0 != row) fail("tiles out of order", tile.r0, row);
    if (tile.r1 <= tile.r0) fail("empty tile", tile.r0, tile.r1);
    if (tile.r1 - tile.r0 > max_rows) fail("tile rows > limit", tile.r1 - tile.r0, max_rows);
    if (tile.k0 != p.ptr[tile.r0] || tile.k1 != p.ptr[tile.r1]) fail("tile entries do not match its rows", tile.k0, tile.k1);
    for (int r = tile.r0; r < tile.r1; ++r) {
      if (p.ptr[r + 1] - p.ptr[r] > kCap) fail("long row inside a short tile", r, p.ptr[r + 1] - p.ptr[r]);
      if (lanes == 1 && tile.r1 - tile.r0 > 1 && p.ptr[r + 1] - p.ptr[r] > kWarpRowMin) {
        fail("warp row shares its tile", r, p.ptr[r + 1] - p.ptr[r]);
      }
    }
    // Row pointer and row operand copies.
    const int w0 = tile.r0 & ~3;
    const int bp = ((tile.r1 + 1 + 3) & ~3) - w0;
    const int br = ((tile.r1 + 3) & ~3) - w0;
    if (bp > kRowStride) fail("row pointer copy exceeds the buffer", bp, kRowStride);
    if (br > kRowStride) fail("row operand copy exceeds the buffer", br, kRowStride);
    if (w0 + bp > p.lines + 1 + kPad) fail("row pointer copy beyond the padded array", w0 + bp, p.lines);
    if (w0 + br > p.lines + kPad) fail("row operand copy beyond the padded vectors", w0 + br, p.lines);
    row = tile.r1;
  }
  if (row != p.lines) fail("tiles do not cover every line", row, p.lines);
  if (chunk != nchunks) fail("chunk count", chunk, nchunks);
  if (li != longs.size()) fail("long rows", static_cast<long long>(li), static_cast<long long>(longs.size()));
}

void check_windows(const Pattern& p, const std::vector<Tile>& tiles, int wmax) {
  std::vector<int> tile_win;
  std::vector<int2> windows;
  const long long covered = build_windows(tiles, p.idx.data(), p.extent, wmax, &tile_win, &windows);
  if (tile_win.size() != tiles.size()) fail("one window id per tile", static_cast<long long>(tile_win.size()), static_cast<long long>(tiles.size()));
  const int ext4 = (p.extent + 3) & ~3;
  for (const int2& w : windows) {
    if (w.x % 4 != 0 || w.y % 4 != 0) fail("window not on 4-element bounds", w.x, w.y);
    if (w.y <= 0 || w.y > wmax) fail("window length", w.y, wmax);
    if (w.x < 0 || w.x + w.y > ext4) fail("window beyond the padded vector", w.x, w.y);
  }
  long long count = 0;
  for (size_t t = 0; t < tiles.size(); ++t) {
    const int id = tile_win[t];
    if (id < -1 || id >= static_cast<int>(windows.size())) {
      fail("window id", id, static_cast<long long>(windows.size()));
      continue;
    }
    if (id < 0) continue;
    const int2 w = windows[static_cast<size_t>(id)];
    for (int k = tiles[t].k0; k < tiles[t].k1; ++k) {
      if (p.idx[static_cast<size_t>(k)] >= w.x && p.idx[static_cast<size_t>(k)] < w.x + w.y) ++count;
    }
  }
  if (wmax <= 0 && !windows.empty()) fail("windows without capacity", static_cast<long long>(windows.size()), wmax);
  if (count != covered) fail("staged count", covered, count);
}

// The chunk plan of an FP32 step pass for pattern p (see plan_chunks).
void check_chunk_plan(const Pattern& p, int wmax, int grid, double split_min) {
  const int cap = kChunkCapF;
  const int round_cap = (kChunkThreads / 32) * kChunkCapF;
  const ChunkPlan P = plan_chunks(p.ptr, p.idx.data(), p.lines, p.extent, cap, wmax, grid, 4,
                                  split_min, 0.999, round_cap);
  if (P.error) fail("plan_chunks reported an error", p.lines, wmax);
  const long long nnz = p.ptr[p.lines];
  const std::vector<int>& ptr = P.split ? P.ptr : p.ptr;
  const std::vector<int>& idx = P.split ? P.idx : p.idx;
  if (static_cast<int>(ptr.size()) != p.lines + 1) fail("main row pointers", static_cast<long long>(ptr.size()), p.lines);
  // Chunks.
  int row = 0, piece = 0;
  size_t li = 0;
  const long long T = static_cast<long long>(P.chunks.size());
  for (long long c = 0; c < T; ++c) {
    const Tile& ch = P.chunks[static_cast<size_t>(c)];
    if (ch.k1 - ch.k0 > cap || ch.k0 > ch.k1) fail("chunk entries", ch.k0, ch.k1);
    if (ch.r1 < 0) {
      if (li >= P.longs.size() || P.longs[li].row != ch.r0) fail("piece without its long row", ch.r0, static_cast<long long>(li));
      if (-ch.r1 - 1 != piece) fail("piece slot order", -ch.r1 - 1, piece);
      if (ch.r0 != row) fail("piece row", ch.r0, row);
      ++piece;
      if (ch.k1 == ptr[static_cast<size_t>(row) + 1]) {
        if (li < P.longs.size() && P.longs[li].chunk0 + P.longs[li].nchunks != piece) fail("long row pieces", P.longs[li].nchunks, piece);
        ++li;
        ++row;
      }
      continue;
    }
    if (ch.r0 != row) fail("chunks out of order", ch.r0, row);
    if (ch.r1 <= ch.r0 || ch.r1 - ch.r0 > kChunkRows) fail("chunk rows", ch.r0, ch.r1);
    if (ch.k0 != ptr[static_cast<size_t>(ch.r0)] || ch.k1 != ptr[static_cast<size_t>(ch.r1)]) fail("chunk entries do not match its rows", ch.k0, ch.k1);
    row = ch.r1;
  }
  if (row != p.lines) fail("chunks do not cover every line", row, p.lines);
  if (piece != P.npieces || li != P.longs.size()) fail("piece count", piece, P.npieces);
  // Segments: every block's in order, together every chunk once.
  if (static_cast<int>(P.seg_start.size()) != grid + 1) fail("segment starts", static_cast<long long>(P.seg_start.size()), grid + 1);
  long long next = 0, inside = 0;
  const int ext4 = (p.extent + 3) & ~3;
  std::vector<int> chunk_block(static_cast<size_t>(T), -1);
  for (int b = 0; b < grid; ++b) {
    for (int s = P.seg_start[b]; s < P.seg_start[b + 1]; ++s) {
      const ChunkSeg& sg = P.segs[static_cast<size_t>(s)];
      if (sg.c0 != next || sg.c1 <= sg.c0 || sg.c1 > T) fail("segment chunks", sg.c0, next);
      if (sg.len > 0) {
        if (sg.lo % 4 != 0 || sg.len % 4 != 0) fail("window not on 4-element bounds", sg.lo, sg.len);
        if (sg.lo < 0 || sg.lo + sg.len > ext4 || sg.lo + sg.len > p.extent + kPad) fail("window beyond the padded vector", sg.lo, sg.len);
        if (sg.len > P.wmax || P.wmax > std::max(wmax, ext4)) fail("window length", sg.len, P.wmax);
      }
      for (int c = sg.c0; c < sg.c1 && c < T; ++c) {
        chunk_block[static_cast<size_t>(c)] = b;
        const Tile& ch = P.chunks[static_cast<size_t>(c)];
        for (int k = ch.k0; k < ch.k1; ++k) {
          const bool in = sg.len > 0 && static_cast<unsigned>(idx[static_cast<size_t>(k)] - sg.lo) < static_cast<unsigned>(sg.len);
          inside += in;
          // A split layout's main entries in a windowed chunk are all inside the window.
          if (P.split && sg.len > 0 && ch.r1 >= 0 && !in) fail("main entry outside its window", k, idx[static_cast<size_t>(k)]);
        }
      }
      next = sg.c1;
    }
  }
  if (next != T) fail("segments do not cover every chunk", next, T);
  if (nnz > 0 && std::abs(static_cast<double>(inside) / static_cast<double>(nnz) - P.staged) > 1e-12) {
    fail("staged share", inside, nnz);
  }
  if (!P.split) {
    if (!P.orounds.empty() || !P.oidx.empty()) fail("outer part of an unsplit layout", static_cast<long long>(P.oidx.size()), 0);
    return;
  }
  // Split: main and outer entries partition the layout's entries, in row order.
  if (static_cast<long long>(P.map.size() + P.omap.size()) != nnz) fail("split entry count", static_cast<long long>(P.map.size() + P.omap.size()), nnz);
  std::vector<char> seen(static_cast<size_t>(nnz), 0);
  for (size_t k = 0; k < P.map.size(); ++k) {
    const int f = P.map[k];
    if (f < 0 || f >= nnz || seen[static_cast<size_t>(f)]++ || P.idx[k] != p.idx[static_cast<size_t>(f)]) fail("main map", static_cast<long long>(k), f);
  }
  for (size_t k = 0; k < P.omap.size(); ++k) {
    const int f = P.omap[k];
    if (f < 0 || f >= nnz || seen[static_cast<size_t>(f)]++ || P.oidx[k] != p.idx[static_cast<size_t>(f)]) fail("outer map", static_cast<long long>(k), f);
  }
  for (int r = 0; r < p.lines; ++r) {
    const int full = p.ptr[r + 1] - p.ptr[r];
    const int parts = (P.ptr[r + 1] - P.ptr[r]) + (P.optr[r + 1] - P.optr[r]);
    if (full != parts) fail("row split", r, full - parts);
  }
  // Outer rounds: every row once, in order, by the block whose chunks hold it.
  if (static_cast<int>(P.oround_start.size()) != grid + 1) fail("round starts", static_cast<long long>(P.oround_start.size()), grid + 1);
  std::vector<int> row_block(static_cast<size_t>(p.lines), -1);
  int orow = 0;
  for (int b = 0; b < grid; ++b) {
    for (int q = P.oround_start[b]; q < P.oround_start[b + 1]; ++q) {
      const int2 rr = P.orounds[static_cast<size_t>(q)];
      if (rr.x != orow || rr.y <= rr.x) fail("outer rounds out of order", rr.x, orow);
      if (P.optr[rr.y] - P.optr[rr.x] > round_cap) fail("outer round exceeds the staging space", P.optr[rr.y] - P.optr[rr.x], round_cap);
      for (int r = rr.x; r < rr.y && r < p.lines; ++r) row_block[static_cast<size_t>(r)] = b;
      orow = rr.y;
    }
  }
  if (orow != p.lines) fail("outer rounds do not cover every row", orow, p.lines);
  for (long long c = 0; c < T; ++c) {
    const Tile& ch = P.chunks[static_cast<size_t>(c)];
    if (ch.r1 < 0) continue;
    for (int r = ch.r0; r < ch.r1; ++r) {
      if (row_block[static_cast<size_t>(r)] != chunk_block[static_cast<size_t>(c)]) fail("outer sum written by another block", r, chunk_block[static_cast<size_t>(c)]);
    }
  }
}

// A pattern from a file: int32 lines, int32 extent, int32 ptr[lines + 1], int32 idx[nnz].
bool read_pattern(const char* path, Pattern* p) {
  std::FILE* f = std::fopen(path, "rb");
  if (f == nullptr) return false;
  int head[2];
  bool ok = std::fread(head, sizeof(int), 2, f) == 2 && head[0] >= 0 && head[1] > 0;
  if (ok) {
    p->lines = head[0];
    p->extent = head[1];
    p->ptr.resize(static_cast<size_t>(p->lines) + 1);
    ok = std::fread(p->ptr.data(), sizeof(int), p->ptr.size(), f) == p->ptr.size() &&
         p->ptr[0] == 0 && p->ptr[static_cast<size_t>(p->lines)] >= 0;
  }
  if (ok) {
    p->idx.resize(static_cast<size_t>(p->ptr[static_cast<size_t>(p->lines)]));
    ok = std::fread(p->idx.data(), sizeof(int), p->idx.size(), f) == p->idx.size();
  }
  std::fclose(f);
  return ok;
}

// The layouts the engine builds for a real pattern: lanes 1 with the FP64 block size and
// the FP32 lane rule with the FP32 block size, at the window capacities of both.
int check_file(const char* path) {
  Pattern p;
  if (!read_pattern(path, &p)) {
    std::printf("FAIL: cannot read %s\n", path);
    return 1;
  }
  const double avg = p.lines > 0 ? static_cast<double>(p.ptr[static_cast<size_t>(p.lines)]) / p.lines : 1.0;
  const int layouts[2][2] = {{1, kTileThreads}, {wide_lanes(avg, kWideThreads), kWideThreads}};
  long long chunks = 0;
  for (const auto& l : layouts) {
    std::vector<Tile> tiles;
    std::vector<LongRow> longs;
    int nchunks = 0;
    build_tiles(p.ptr, p.lines, l[0], l[1], &tiles, &longs, &nchunks);
    check_tiles(p, l[0], l[1], tiles, longs, nchunks);
    for (int wmax : {0, 16384, 40960}) check_windows(p, tiles, wmax);
    chunks += nchunks;
  }
  for (int wmax : {0, 32768}) check_chunk_plan(p, wmax, 152, 0.5);
  if (g_failures != 0) {
    std::printf("%d failures\n", g_failures);
    return 1;
  }
  std::printf("OK %d lines, %d nonzeros, %lld chunk tiles\n", p.lines, p.ptr[static_cast<size_t>(p.lines)], chunks);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1) return check_file(argv[1]);
  // The FP32 lane rule: two lanes per 10-entry column, four per 20-entry row, and never more
  // rows per tile than a tile can stage.
  if (wide_lanes(10.0, kWideThreads) != 2) fail("wide_lanes(10)", wide_lanes(10.0, kWideThreads), 2);
  if (wide_lanes(20.0, kWideThreads) != 4) fail("wide_lanes(20)", wide_lanes(20.0, kWideThreads), 4);
  for (double avg = 0.5; avg < 5000.0; avg *= 1.37) {
    const int lanes = wide_lanes(avg, kWideThreads);
    if (lanes < 1 || lanes > 32 || (lanes & (lanes - 1)) != 0) fail("wide_lanes power of two", lanes, 0);
    if (kWideThreads / lanes > kMaxTileRows) fail("wide_lanes rows", kWideThreads / lanes, kMaxTileRows);
  }
  // Step graphs: two kernels per step, four evaluation kernels after every kEvalStride steps
  // and after the last.
  if (graph_kernel_launches(1) != 6) fail("graph launches (1)", graph_kernel_launches(1), 6);
  if (graph_kernel_launches(kEvalStride) != 2 * kEvalStride + 4) fail("graph launches (stride)", graph_kernel_launches(kEvalStride), 2 * kEvalStride + 4);
  if (graph_kernel_launches(32) != 64 + 4 * ((32 + kEvalStride - 1) / kEvalStride)) fail("graph launches (32)", graph_kernel_launches(32), 0);

  int layouts = 0;
  for (unsigned seed = 1; seed <= 3; ++seed) {
    for (int banded = 0; banded < 2; ++banded) {
      const Pattern p = make_pattern(seed * 7919u + banded, 4000 + 37 * static_cast<int>(seed), 30001 + static_cast<int>(seed), banded != 0);
      for (int threads : {kTileThreads, kWideThreads}) {
        for (int lanes = 1; lanes <= 32; lanes *= 2) {
          std::vector<Tile> tiles;
          std::vector<LongRow> longs;
          int nchunks = 0;
          build_tiles(p.ptr, p.lines, lanes, threads, &tiles, &longs, &nchunks);
          check_tiles(p, lanes, threads, tiles, longs, nchunks);
          for (int wmax : {0, 1024, 8192, 40000}) check_windows(p, tiles, wmax);
          ++layouts;
        }
      }
      // The FP32 chunk plans: unstaged, windowed and split forms, and grids larger than the
      // number of chunks.
      for (int wmax : {0, 1024, 4096, 8192, 32768}) {
        for (int grid : {1, 7, 152, 4000}) {
          for (double split_min : {0.0, 0.5}) check_chunk_plan(p, wmax, grid, split_min);
          ++layouts;
        }
      }
    }
  }
  if (g_failures != 0) {
    std::printf("%d failures\n", g_failures);
    return 1;
  }
  std::printf("OK %d layouts\n", layouts);
  return 0;
}

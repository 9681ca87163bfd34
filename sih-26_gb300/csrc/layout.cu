// layout.cu -- host planning of the step passes' chunk layouts (see chunks.cuh).
//
// plan_chunks() takes one layout of the matrix (the CSR copy for the row pass, the CSC copy
// for the column pass) and decides, once at load time:
//   * the chunks (rows cut at kChunkRows rows and `cap` entries, long rows into pieces);
//   * each chunk's window of the gathered vector (build_windows, the same rule as the tile
//     layouts), and from the share of entries the windows hold whether the layout stages
//     windows at all, stages them over every entry, or is SPLIT into a main part gathered
//     from windows only and an outer part gathered from L2;
//   * which chunks each block of the grid owns (a cost model: entries plus a fixed cost per
//     window staged), the block's segments, and for a split layout the block's outer chunks.
// Everything here is plain host code: the engine uploads the result, and
// tests/host/layout_check.cu checks it on the CPU.
#include "engine.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>

namespace sgb {

namespace {

// Consecutive rows while the chunk has at most kChunkRows rows and `cap` entries, and every
// row of it shares `row_win` (nullptr: no window constraint); a row longer than `cap` becomes
// pieces of `cap` entries, listed as a LongRow.
void cut_chunks(const std::vector<int>& ptr, int r_begin, int r_end, int cap,
                const std::vector<int>* row_win, std::vector<Tile>* chunks,
                std::vector<LongRow>* longs, int* npieces) {
  int r = r_begin;
  while (r < r_end) {
    const int len = ptr[r + 1] - ptr[r];
    if (len > cap) {
      LongRow lr{r, *npieces, 0};
      for (int k = ptr[r]; k < ptr[r + 1]; k += cap) {
        const int k1 = std::min(k + cap, ptr[r + 1]);
        chunks->push_back(Tile{r, -(*npieces) - 1, k, k1});
        ++*npieces;
        ++lr.nchunks;
      }
      longs->push_back(lr);
      ++r;
      continue;
    }
    const int begin = r;
    const int w = row_win ? (*row_win)[r] : 0;
    ++r;
    while (r < r_end && r - begin < kChunkRows && ptr[r + 1] - ptr[r] <= cap &&
           ptr[r + 1] - ptr[begin] <= cap && (row_win == nullptr || (*row_win)[r] == w)) {
      ++r;
    }
    chunks->push_back(Tile{begin, r, ptr[begin], ptr[r]});
  }
}

// The start lo (a multiple of 4, within [0, ext4 - wmax]) for which [lo, lo + wmax) holds the
// most of the sorted indices v, centred among the starts that do; *count receives that most.
int best_start(const std::vector<int>& v, int wmax, int ext4, int* count) {
  int best = 0, bl = 0, br = 0;
  for (int r = 0, l = 0; r < static_cast<int>(v.size()); ++r) {
    while (v[r] - v[l] >= wmax) ++l;
    if (r - l + 1 > best) {
      best = r - l + 1;
      bl = l;
      br = r;
    }
  }
  *count = best;
  long long lo = 0;
  if (best > 0) {
    const long long lo_min = static_cast<long long>(v[br]) - wmax + 1, lo_max = v[bl];
    lo = lo_min + (lo_max - lo_min) / 2;
  }
  lo = std::max(0LL, std::min(lo, static_cast<long long>(ext4 - wmax)));
  return static_cast<int>(lo) & ~3;
}

int held_by(const Tile& t, const int* idx, int lo, int len) {
  int held = 0;
  for (int k = t.k0; k < t.k1; ++k) {
    held += static_cast<unsigned>(idx[k] - lo) < static_cast<unsigned>(len);
  }
  return held;
}

// Windows of a chunk sequence, in chunk order. A chunk keeps the window its block holds
// while that window holds all but 2% of what the chunk's own best window would. Otherwise the
// window that best serves the next kLookahead chunks together is weighed against the one held
// over those chunks, and replaces it only if it holds 3% more of their entries: a chunk's own
// best window is tuned to its few scattered entries, and restaging costs a block barrier and
// a copy of the whole window, so a window changes only where the pattern moves (a new period
// of a block-angular matrix, say). A chunk whose best window holds fewer than 1/8 of its
// entries gathers from global memory. Returns the entries that fall inside their chunk's
// window.
long long plan_windows(const std::vector<Tile>& chunks, const int* idx, int extent, int wmax,
                       std::vector<int>* chunk_win, std::vector<int2>* windows) {
  constexpr int kLookahead = 32;
  const int nchunks = static_cast<int>(chunks.size());
  chunk_win->assign(static_cast<size_t>(nchunks), -1);
  windows->clear();
  if (wmax <= 0 || nchunks == 0 || extent <= 0) return 0;
  const int ext4 = (extent + 3) & ~3;
  long long covered = 0;
  if (ext4 <= wmax) {  // the whole vector fits: one window for every chunk
    windows->push_back(make_int2(0, ext4));
    chunk_win->assign(static_cast<size_t>(nchunks), 0);
    for (const Tile& t : chunks) covered += t.k1 - t.k0;
    return covered;
  }
  std::vector<int> v;
  int current = -1;
  int weighed_until = 0;  // the held window was last weighed over the chunks before this one
  for (int c = 0; c < nchunks; ++c) {
    const Tile& tl = chunks[static_cast<size_t>(c)];
    const int entries = tl.k1 - tl.k0;
    if (entries == 0) {
      (*chunk_win)[static_cast<size_t>(c)] = current;
      continue;
    }
    v.assign(idx + tl.k0, idx + tl.k1);
    std::sort(v.begin(), v.end());
    int best = 0;
    best_start(v, wmax, ext4, &best);
    if (best * 8 < entries) continue;  // gathers from global memory
    const int2 cw = current >= 0 ? (*windows)[static_cast<size_t>(current)] : make_int2(0, 0);
    const int held = current >= 0 ? held_by(tl, idx, cw.x, cw.y) : 0;
    // Within the chunks a weighing already covered, only a collapse of the held share
    // brings the window up again.
    if (current >= 0 && (held >= best - 0.02 * entries || (c < weighed_until && 2 * held >= best))) {
      (*chunk_win)[static_cast<size_t>(c)] = current;
      continue;
    }
    // The window that best serves this chunk and the next ones together.
    const int c_end = std::min(nchunks, c + kLookahead);
    v.clear();
    for (int d = c; d < c_end; ++d) {
      v.insert(v.end(), idx + chunks[static_cast<size_t>(d)].k0,
               idx + chunks[static_cast<size_t>(d)].k1);
    }
    std::sort(v.begin(), v.end());
    int union_best = 0;
    const int lo = best_start(v, wmax, ext4, &union_best);
    if (current >= 0) {
      long long held_cur = 0, held_new = 0;
      for (int d = c; d < c_end; ++d) {
        held_cur += held_by(chunks[static_cast<size_t>(d)], idx, cw.x, cw.y);
        held_new += held_by(chunks[static_cast<size_t>(d)], idx, lo, wmax);
      }
      if (static_cast<double>(held_new) <= held_cur + 0.03 * static_cast<double>(v.size())) {
        (*chunk_win)[static_cast<size_t>(c)] = current;
        weighed_until = c_end;
        continue;
      }
    }
    weighed_until = c_end;
    windows->push_back(make_int2(lo, wmax));
    current = static_cast<int>(windows->size()) - 1;
    (*chunk_win)[static_cast<size_t>(c)] = current;
  }
  for (int c = 0; c < nchunks; ++c) {
    const int w = (*chunk_win)[static_cast<size_t>(c)];
    if (w < 0) continue;
    const int2 r = (*windows)[static_cast<size_t>(w)];
    covered += held_by(chunks[static_cast<size_t>(c)], idx, r.x, r.y);
  }
  return covered;
}

}  // namespace

ChunkPlan plan_chunks(const std::vector<int>& ptr, const int* idx, int lines, int extent, int cap,
                      int wmax, int grid, int elem_bytes, double split_min, double full_min,
                      int outer_round_cap) {
  ChunkPlan p;
  p.cap = cap;
  p.grid = std::max(1, grid);
  const long long nnz = lines > 0 ? ptr[lines] : 0;
  // Base chunks over the whole layout and their windows.
  std::vector<Tile> base;
  std::vector<LongRow> base_longs;
  int base_pieces = 0;
  cut_chunks(ptr, 0, lines, cap, nullptr, &base, &base_longs, &base_pieces);
  std::vector<int> tile_win;
  std::vector<int2> windows;
  long long covered = 0;
  if (wmax > 0 && nnz > 0) {
    covered = plan_windows(base, idx, extent, wmax, &tile_win, &windows);
  } else {
    tile_win.assign(base.size(), -1);
  }
  const double share = nnz > 0 ? static_cast<double>(covered) / static_cast<double>(nnz) : 0.0;
  p.coverage = share;
  std::vector<int> chunk_win;
  if (windows.empty() || share < split_min) {
    // No staging: every gather from L2.
    p.chunks = base;
    p.longs = base_longs;
    p.npieces = base_pieces;
    chunk_win.assign(p.chunks.size(), -1);
    windows.clear();
    p.staged = 0.0;
  } else if (share >= full_min) {
    p.chunks = base;
    p.longs = base_longs;
    p.npieces = base_pieces;
    chunk_win = tile_win;
    p.staged = share;
  } else {
    // Split: a row's window is its base chunk's; long rows keep every entry in the main part
    // and gather from global memory.
    p.split = true;
    std::vector<int> row_win(static_cast<size_t>(lines), -1);
    for (size_t t = 0; t < base.size(); ++t) {
      const Tile& tl = base[t];
      if (tl.r1 < 0) continue;
      for (int r = tl.r0; r < tl.r1; ++r) row_win[r] = tile_win[t];
    }
    p.ptr.assign(static_cast<size_t>(lines) + 1, 0);
    p.optr.assign(static_cast<size_t>(lines) + 1, 0);
    long long in_window = 0;
    for (int r = 0; r < lines; ++r) {
      const int w = row_win[r];
      const int lo = w >= 0 ? windows[w].x : 0, len = w >= 0 ? windows[w].y : 0;
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
        const bool inside = w < 0 || static_cast<unsigned>(idx[k] - lo) < static_cast<unsigned>(len);
        if (inside) {
          p.idx.push_back(idx[k]);
          p.map.push_back(k);
          in_window += w >= 0;
        } else {
          p.oidx.push_back(idx[k]);
          p.omap.push_back(k);
        }
      }
      p.ptr[r + 1] = static_cast<int>(p.idx.size());
      p.optr[r + 1] = static_cast<int>(p.oidx.size());
    }
    cut_chunks(p.ptr, 0, lines, cap, &row_win, &p.chunks, &p.longs, &p.npieces);
    chunk_win.resize(p.chunks.size());
    for (size_t c = 0; c < p.chunks.size(); ++c) {
      const Tile& tl = p.chunks[c];
      chunk_win[c] = tl.r1 < 0 ? -1 : row_win[tl.r0];
    }
    p.staged = nnz > 0 ? static_cast<double>(in_window) / static_cast<double>(nnz) : 0.0;
  }
  // Window capacity actually used.
  p.wmax = 0;
  for (const int2& w : windows) p.wmax = std::max(p.wmax, w.y);

  // Blocks: cut the chunk sequence where the running cost reaches the average. A chunk costs
  // its entries plus a fixed overhead; staging a window costs its bytes / 32 entries (it is
  // copied from L2 at a multiple of the matrix stream's speed).
  const int G = p.grid;
  const long long T = static_cast<long long>(p.chunks.size());
  const double per_chunk = 16.0;
  const double stage_cost = static_cast<double>(p.wmax) * elem_bytes / 32.0;
  double total = 0.0;
  long long stages = 0;
  for (long long c = 0; c < T; ++c) {
    total += (p.chunks[c].k1 - p.chunks[c].k0) + per_chunk;
    if (chunk_win[c] >= 0 && (c == 0 || chunk_win[c] != chunk_win[c - 1])) ++stages;
  }
  const double target = (total + stage_cost * static_cast<double>(stages + G)) / G;
  std::vector<long long> bstart(static_cast<size_t>(G) + 1, T);
  bstart[0] = 0;
  {
    int b = 0;
    double acc = 0.0;
    int held = -2;  // the window the current block holds (-2: none yet)
    for (long long c = 0; c < T; ++c) {
      if (chunk_win[c] >= 0 && chunk_win[c] != held) acc += stage_cost;
      held = chunk_win[c] >= 0 ? chunk_win[c] : held;
      acc += (p.chunks[c].k1 - p.chunks[c].k0) + per_chunk;
      if (acc >= target && b + 1 < G && c + 1 < T) {
        bstart[++b] = c + 1;
        acc = 0.0;
        held = -2;
      }
    }
    for (int q = b + 1; q <= G; ++q) bstart[q] = T;
  }
  // Segments.
  p.seg_start.assign(static_cast<size_t>(G) + 1, 0);
  for (int b = 0; b < G; ++b) {
    p.seg_start[b] = static_cast<int>(p.segs.size());
    long long c = bstart[b];
    while (c < bstart[b + 1]) {
      long long e = c + 1;
      while (e < bstart[b + 1] && chunk_win[e] == chunk_win[c]) ++e;
      ChunkSeg sg{static_cast<int>(c), static_cast<int>(e), 0, 0};
      if (chunk_win[c] >= 0) {
        sg.lo = windows[chunk_win[c]].x;
        sg.len = windows[chunk_win[c]].y;
      }
      p.segs.push_back(sg);
      c = e;
    }
  }
  p.seg_start[G] = static_cast<int>(p.segs.size());
  // Outer rounds: block b sums the outer entries of rows [row_begin[b], row_begin[b + 1]),
  // where row_begin[b] is the first row of its first chunk. Its main chunks lie inside that
  // range (a piece of a long row may not, but pieces read no outer sum), and every row of it
  // is written, zero where it has no outer entry. A round is a run of those rows whose outer
  // entries fit the block's staging space (outer_round_cap entries).
  if (p.split) {
    std::vector<int> row_begin(static_cast<size_t>(G) + 1, lines);
    for (int b = 0; b < G; ++b) row_begin[b] = bstart[b] < T ? p.chunks[bstart[b]].r0 : lines;
    p.oround_start.assign(static_cast<size_t>(G) + 1, 0);
    for (int b = 0; b < G; ++b) {
      p.oround_start[b] = static_cast<int>(p.orounds.size());
      int r = row_begin[b];
      while (r < row_begin[b + 1]) {
        int e = r;
        while (e < row_begin[b + 1] && p.optr[e + 1] - p.optr[r] <= outer_round_cap) ++e;
        if (e == r) {  // one row with more outer entries than the staging space holds
          std::fprintf(stderr, "plan_chunks: row %d has %d outer entries (> %d)\n", r,
                       p.optr[r + 1] - p.optr[r], outer_round_cap);
          p.error = true;
          break;
        }
        p.orounds.push_back(make_int2(r, e));
        r = e;
      }
    }
    p.oround_start[G] = static_cast<int>(p.orounds.size());
    if (row_begin[0] != 0) p.error = true;
  }
  if (std::getenv("SANKHYA_GB300_LAYOUT_LOG") != nullptr) {
    std::fprintf(stderr,
                 "plan_chunks: %d lines, %lld entries, cap %d, wmax %d: coverage %.4f, %s, "
                 "staged %.4f, %zu chunks, %zu windows, %zu segments, %zu outer entries, "
                 "%zu outer rounds, %d pieces\n",
                 lines, nnz, cap, p.wmax, p.coverage,
                 p.split ? "split" : (p.wmax > 0 ? "windowed" : "unstaged"), p.staged,
                 p.chunks.size(), windows.size(), p.segs.size(), p.oidx.size(),
                 p.orounds.size(), p.npieces);
  }
  return p;
}

}  // namespace sgb

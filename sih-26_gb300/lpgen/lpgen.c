/*
 * lpgen.c -- seeded synthetic LPs with a planted optimum.
 *
 * Every generator draws a point x0 inside the column box, a multiplier vector lambda and
 * reduced costs z that are complementary to x0 (z_j >= 0 where x0_j sits at its lower bound,
 * z_j <= 0 at its upper bound, 0 strictly inside), then sets the row bounds from A x0 and the
 * cost to c = A^T lambda + z. (x0, lambda) satisfies the KKT conditions of
 *     min c^T x  s.t.  rl <= A x <= ru,  l <= x <= u
 * by construction, so f* = c^T x0 is known without solving anything.
 *
 * Shapes:
 *   lpgen_planted_uniform  m x n, exactly k distinct uniform rows per column, N(0,1) values,
 *                          equality rows, 0 <= x <= 10; x0: 30% at 0, 10% at 10, the rest
 *                          U(0.1, 9.9); lambda ~ N(0,1); z ~ +-U(0.1, 1) at the bounds.
 *   lpgen_planted_blocks   block-angular multi-period structure: B blocks of R rows x C cols,
 *                          k distinct uniform rows per column inside its block plus one +-1
 *                          linking entry into a uniform row of the next block (none for the
 *                          last block); otherwise as planted_uniform.
 *   lpgen_planted_zipf     load-balance stress: row lengths from a Zipf law (P(L) ~ L^-a,
 *                          drawn as min_len U^(-1/(a-1)) and clipped to [min_len, max_len]),
 *                          scaled so the lengths sum to about target_nnz, distinct uniform
 *                          columns per row, values +-10^U(-3,3) (log-uniform magnitude over
 *                          [1e-3, 1e3], random sign), 0 <= x <= 10, equality rows.
 *   lpgen_planted_nondegenerate  as planted_uniform, but with a unique and nondegenerate
 *                          optimum: exactly m basic columns (x0 in U(0.1, 9.9), z = 0), the
 *                          p-th of which has an entry of magnitude 1 + |N(0,1)| in row p (so
 *                          the basis matrix has a heavy diagonal and is nonsingular); every
 *                          other column sits at 0 or 10 with |z| in U(0.1, 1). x*, y* are then
 *                          differentiable in c, b and the bounds.
 *   lpgen_planted_general  every row kind (equality, one-sided active/slack, range active at
 *                          either side, free) and every column kind (boxed, lower-only,
 *                          upper-only, free, fixed) for parity coverage.
 *
 * Output arrays are caller-allocated; lpgen_*_nnz gives the size to allocate. The CSC layout
 * (int32 column starts, ascending int32 row indices, FP64 values) is the one SANKHYA's Model
 * holds. Randomness is MT19937-64 (Matsumoto & Nishimura 2000) seeded per instance; log and
 * cos are computed from IEEE basic operations only, so an instance is bit-identical on
 * every host.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int32_t rows, cols;
  int64_t nnz;
  int32_t* col_starts;
  int32_t* row_index;
  double* values;
  double* col_cost;
  double* col_lower;
  double* col_upper;
  double* row_lower;
  double* row_upper;
  double* x0;     /* planted primal point (cols) */
  double* lambda; /* planted row multipliers, c = A^T lambda + z (rows) */
  double fstar;   /* c^T x0 */
} lpgen_lp;

/* ---- MT19937-64 ---------------------------------------------------------------------- */
typedef struct {
  uint64_t mt[312];
  int index;
} mt64;

static void mt64_seed(mt64* g, uint64_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 312; ++i) {
    g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
  }
  g->index = 312;
}

static uint64_t mt64_next(mt64* g) {
  if (g->index >= 312) {
    for (int i = 0; i < 312; ++i) {
      const uint64_t x = (g->mt[i] & 0xFFFFFFFF80000000ULL) | (g->mt[(i + 1) % 312] & 0x7FFFFFFFULL);
      g->mt[i] = g->mt[(i + 156) % 312] ^ (x >> 1) ^ ((x & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
    }
    g->index = 0;
  }
  uint64_t x = g->mt[g->index++];
  x ^= (x >> 29) & 0x5555555555555555ULL;
  x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
  x ^= (x << 37) & 0xFFF7EEE000000000ULL;
  x ^= (x >> 43);
  return x;
}

/* [0, 1) with 53 random bits. */
static double unif(mt64* g) { return (double)(mt64_next(g) >> 11) * (1.0 / 9007199254740992.0); }
static double unif_ab(mt64* g, double a, double b) { return a + (b - a) * unif(g); }
/* Uniform integer in [0, k), k < 2^32, by the multiply-shift map of the top 32 bits. */
static int32_t unif_int(mt64* g, int32_t k) {
  return (int32_t)(((mt64_next(g) >> 32) * (uint64_t)k) >> 32);
}
/* log and cos from +, -, *, / and frexp only (all exactly specified by IEEE 754), so the
 * same seed gives the same LP on x86-64 and aarch64 whatever their libm does.
 * log: x = m 2^e with m in [1/sqrt2, sqrt2), log m = 2 atanh(s), s = (m-1)/(m+1).
 * cos: reduce to [0, pi/4] by the symmetries of cos, then the Taylor series. */
static double det_log(double x) {
  int e;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    e -= 1;
  }
  const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
  double term = s, sum = 0.0;
  for (int k = 1; k < 41; k += 2) {
    sum += term / (double)k;
    term *= s2;
  }
  return 2.0 * sum + (double)e * 0.69314718055994530942;
}

static double taylor_cos(double t) { /* |t| <= pi/4 */
  const double t2 = t * t;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; ++k) {
    term *= -t2 / (double)((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}

static double taylor_sin(double t) { /* |t| <= pi/4 */
  const double t2 = t * t;
  double term = t, sum = t;
  for (int k = 1; k < 14; ++k) {
    term *= -t2 / (double)((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}

/* cos(2 pi u) for u in [0, 1). */
static double det_cos_turns(double u) {
  const double two_pi = 6.283185307179586476925;
  double w = u < 0.5 ? u : 1.0 - u; /* cos is even and 1-periodic in turns: w in [0, 0.5] */
  double sign = 1.0;
  if (w > 0.25) { /* cos(2 pi w) = -cos(2 pi (0.5 - w)) */
    w = 0.5 - w;
    sign = -1.0;
  }
  if (w <= 0.125) return sign * taylor_cos(two_pi * w);
  return sign * taylor_sin(two_pi * (0.25 - w)); /* cos(a) = sin(pi/2 - a) */
}

/* exp from IEEE basic operations and ldexp: x = k ln2 + r with |r| <= ln2 / 2, then the
 * Taylor series of exp(r) (27 terms: far past double precision for |r| <= 0.35). */
static double det_exp(double x) {
  const double ln2 = 0.69314718055994530942;
  const double kf = floor(x / ln2 + 0.5);
  const double r = x - kf * ln2;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 28; ++k) {
    term *= r / (double)k;
    sum += term;
  }
  return ldexp(sum, (int)kf);
}

/* Standard normal by Box-Muller (one value per call). */
static double normal(mt64* g) {
  const double u1 = ((double)(mt64_next(g) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  const double u2 = unif(g);
  return sqrt(-2.0 * det_log(u1)) * det_cos_turns(u2);
}

/* k distinct uniform rows from [base, base + span), sorted ascending, into out. */
static void pick_rows(mt64* g, int32_t base, int32_t span, int32_t k, int32_t* out) {
  for (int32_t t = 0; t < k; ++t) {
    int32_t r;
    int dup;
    do {
      r = base + unif_int(g, span);
      dup = 0;
      for (int32_t s = 0; s < t; ++s) dup |= out[s] == r;
    } while (dup);
    int32_t p = t;
    while (p > 0 && out[p - 1] > r) {
      out[p] = out[p - 1];
      --p;
    }
    out[p] = r;
  }
}

/* x0 and z for a 0 <= x <= 10 column, shared by the uniform and block shapes. */
static void box_point(mt64* g, double* x0, double* z) {
  const double u = unif(g);
  if (u < 0.3) {
    *x0 = 0.0;
    *z = unif_ab(g, 0.1, 1.0);
  } else if (u < 0.4) {
    *x0 = 10.0;
    *z = -unif_ab(g, 0.1, 1.0);
  } else {
    *x0 = unif_ab(g, 0.1, 9.9);
    *z = 0.0;
  }
}

/* b = A x0 into rl = ru; c = A^T lambda + z; f* = c^T x0. */
static void finish_equalities(lpgen_lp* lp, const double* z) {
  for (int32_t i = 0; i < lp->rows; ++i) lp->row_lower[i] = 0.0;
  for (int32_t j = 0; j < lp->cols; ++j) {
    double c = z[j];
    for (int32_t k = lp->col_starts[j]; k < lp->col_starts[j + 1]; ++k) {
      lp->row_lower[lp->row_index[k]] += lp->values[k] * lp->x0[j];
      c += lp->values[k] * lp->lambda[lp->row_index[k]];
    }
    lp->col_cost[j] = c;
  }
  memcpy(lp->row_upper, lp->row_lower, sizeof(double) * (size_t)lp->rows);
  double f = 0.0;
  for (int32_t j = 0; j < lp->cols; ++j) f += lp->col_cost[j] * lp->x0[j];
  lp->fstar = f;
}

int64_t lpgen_planted_uniform_nnz(int32_t m, int32_t n, int32_t k) {
  (void)m;
  return (int64_t)n * k;
}

int32_t lpgen_planted_uniform(int32_t m, int32_t n, int32_t k, uint64_t seed, lpgen_lp* lp) {
  if (m <= 0 || n <= 0 || k <= 0 || k > m) return 1;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  lp->rows = m;
  lp->cols = n;
  lp->nnz = (int64_t)n * k;
  int64_t at = 0;
  for (int32_t j = 0; j < n; ++j) {
    lp->col_starts[j] = (int32_t)at;
    pick_rows(g, 0, m, k, lp->row_index + at);
    for (int32_t t = 0; t < k; ++t) lp->values[at + t] = normal(g);
    at += k;
    box_point(g, &lp->x0[j], &z[j]);
    lp->col_lower[j] = 0.0;
    lp->col_upper[j] = 10.0;
  }
  lp->col_starts[n] = (int32_t)at;
  for (int32_t i = 0; i < m; ++i) lp->lambda[i] = normal(g);
  finish_equalities(lp, z);
  free(z);
  free(g);
  return 0;
}

int64_t lpgen_planted_blocks_nnz(int32_t blocks, int32_t rows_per_block, int32_t cols_per_block,
                                 int32_t k) {
  (void)rows_per_block;
  return (int64_t)blocks * cols_per_block * k + (int64_t)(blocks - 1) * cols_per_block;
}

int32_t lpgen_planted_blocks(int32_t blocks, int32_t rows_per_block, int32_t cols_per_block,
                             int32_t k, uint64_t seed, lpgen_lp* lp) {
  if (blocks <= 0 || rows_per_block <= 0 || cols_per_block <= 0 || k <= 0 || k > rows_per_block) {
    return 1;
  }
  const int64_t m64 = (int64_t)blocks * rows_per_block, n64 = (int64_t)blocks * cols_per_block;
  const int64_t nnz = lpgen_planted_blocks_nnz(blocks, rows_per_block, cols_per_block, k);
  if (m64 > INT32_MAX || n64 > INT32_MAX || nnz > INT32_MAX) return 2;
  const int32_t m = (int32_t)m64, n = (int32_t)n64;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  lp->rows = m;
  lp->cols = n;
  lp->nnz = nnz;
  int64_t at = 0;
  for (int32_t t = 0; t < blocks; ++t) {
    for (int32_t c = 0; c < cols_per_block; ++c) {
      const int32_t j = t * cols_per_block + c;
      lp->col_starts[j] = (int32_t)at;
      pick_rows(g, t * rows_per_block, rows_per_block, k, lp->row_index + at);
      for (int32_t s = 0; s < k; ++s) lp->values[at + s] = normal(g);
      at += k;
      if (t + 1 < blocks) {
        /* The inventory link: one +-1 entry in a row of the next period's block, which lies
         * above every row of this block, so the column stays sorted. */
        lp->row_index[at] = (t + 1) * rows_per_block + unif_int(g, rows_per_block);
        lp->values[at] = unif(g) < 0.5 ? -1.0 : 1.0;
        ++at;
      }
      box_point(g, &lp->x0[j], &z[j]);
      lp->col_lower[j] = 0.0;
      lp->col_upper[j] = 10.0;
    }
  }
  lp->col_starts[n] = (int32_t)at;
  for (int32_t i = 0; i < m; ++i) lp->lambda[i] = normal(g);
  finish_equalities(lp, z);
  free(z);
  free(g);
  return 0;
}

int64_t lpgen_planted_general_nnz(int32_t m, int32_t n, int32_t k) {
  (void)m;
  return (int64_t)n * k;
}

/* flags: bit 0 leaves out free columns, bit 1 leaves out free rows (they become one-sided).
 * SANKHYA's optimality standard multiplies a free column's reduced cost (a free row's
 * multiplier) by an infinite slack, so an LP with either is `optimal` only when that value is
 * exactly zero -- a matter of rounding luck, unfit for comparing two implementations. */
int32_t lpgen_planted_general(int32_t m, int32_t n, int32_t k, int32_t flags, uint64_t seed,
                              lpgen_lp* lp) {
  if (m <= 0 || n <= 0 || k <= 0 || k > m) return 1;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* act = (double*)calloc((size_t)m, sizeof(double));
  lp->rows = m;
  lp->cols = n;
  lp->nnz = (int64_t)n * k;
  const double inf = INFINITY;
  int64_t at = 0;
  for (int32_t j = 0; j < n; ++j) {
    lp->col_starts[j] = (int32_t)at;
    pick_rows(g, 0, m, k, lp->row_index + at);
    for (int32_t t = 0; t < k; ++t) lp->values[at + t] = normal(g);
    at += k;
    double l, u, x, zz = 0.0;
    int kind = unif_int(g, 6);
    if (kind == 3 && (flags & 1)) kind = 1;
    const double state = unif(g);
    switch (kind) {
      case 0: /* boxed, arbitrary interval */
        l = -unif_ab(g, 0.0, 5.0);
        u = l + unif_ab(g, 1.0, 10.0);
        if (state < 0.35) { x = l; zz = unif_ab(g, 0.1, 1.0); }
        else if (state < 0.6) { x = u; zz = -unif_ab(g, 0.1, 1.0); }
        else { x = unif_ab(g, l + 0.05 * (u - l), u - 0.05 * (u - l)); }
        break;
      case 1: /* lower bound only */
        l = unif_ab(g, -5.0, 5.0);
        u = inf;
        if (state < 0.5) { x = l; zz = unif_ab(g, 0.1, 1.0); }
        else { x = l + unif_ab(g, 0.1, 5.0); }
        break;
      case 2: /* upper bound only */
        l = -inf;
        u = unif_ab(g, -5.0, 5.0);
        if (state < 0.5) { x = u; zz = -unif_ab(g, 0.1, 1.0); }
        else { x = u - unif_ab(g, 0.1, 5.0); }
        break;
      case 3: /* free */
        l = -inf;
        u = inf;
        x = 3.0 * normal(g);
        break;
      case 4: /* fixed */
        l = unif_ab(g, -5.0, 5.0);
        u = l;
        x = l;
        zz = normal(g);
        break;
      default: /* the 0 <= x <= 10 box of the uniform shape */
        l = 0.0;
        u = 10.0;
        box_point(g, &x, &zz);
        break;
    }
    lp->col_lower[j] = l;
    lp->col_upper[j] = u;
    lp->x0[j] = x;
    z[j] = zz;
  }
  lp->col_starts[n] = (int32_t)at;
  for (int32_t j = 0; j < n; ++j) {
    for (int32_t q = lp->col_starts[j]; q < lp->col_starts[j + 1]; ++q) {
      act[lp->row_index[q]] += lp->values[q] * lp->x0[j];
    }
  }
  for (int32_t i = 0; i < m; ++i) {
    const double a = act[i];
    double rl, ru, lam = 0.0;
    int row_kind = unif_int(g, 8);
    if (row_kind == 7 && (flags & 2)) row_kind = 2;
    switch (row_kind) {
      case 0: rl = a; ru = a; lam = normal(g); break;
      case 1: rl = a; ru = inf; lam = unif_ab(g, 0.1, 1.0); break;
      case 2: rl = a - unif_ab(g, 0.5, 2.0); ru = inf; break;
      case 3: rl = -inf; ru = a; lam = -unif_ab(g, 0.1, 1.0); break;
      case 4: rl = -inf; ru = a + unif_ab(g, 0.5, 2.0); break;
      case 5: rl = a; ru = a + unif_ab(g, 0.5, 3.0); lam = unif_ab(g, 0.1, 1.0); break;
      case 6: rl = a - unif_ab(g, 0.5, 3.0); ru = a; lam = -unif_ab(g, 0.1, 1.0); break;
      default: rl = -inf; ru = inf; break;
    }
    lp->row_lower[i] = rl;
    lp->row_upper[i] = ru;
    lp->lambda[i] = lam;
  }
  for (int32_t j = 0; j < n; ++j) {
    double c = z[j];
    for (int32_t q = lp->col_starts[j]; q < lp->col_starts[j + 1]; ++q) {
      c += lp->values[q] * lp->lambda[lp->row_index[q]];
    }
    lp->col_cost[j] = c;
  }
  double f = 0.0;
  for (int32_t j = 0; j < n; ++j) f += lp->col_cost[j] * lp->x0[j];
  lp->fstar = f;
  free(act);
  free(z);
  free(g);
  return 0;
}

/* Row lengths of the Zipf shape, drawn first from the instance's generator so that the
 * _nnz query and the generator agree. Returns the total. */
static int64_t zipf_lengths(mt64* g, int32_t m, int32_t n, int64_t target_nnz, double exponent,
                            int32_t min_len, int32_t max_len, int32_t* len) {
  const double inv_tail = 1.0 / (exponent - 1.0);
  double raw_total = 0.0;
  double* raw = (double*)malloc(sizeof(double) * (size_t)m);
  for (int32_t i = 0; i < m; ++i) {
    const double u = ((double)(mt64_next(g) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
    double l = (double)min_len * det_exp(-inv_tail * det_log(u));
    if (l > (double)max_len) l = (double)max_len;
    raw[i] = floor(l);
    raw_total += raw[i];
  }
  const double scale = (double)target_nnz / raw_total;
  const int32_t cap = max_len < n ? max_len : n;
  int64_t total = 0;
  for (int32_t i = 0; i < m; ++i) {
    double l = floor(raw[i] * scale + 0.5);
    if (l < (double)min_len) l = (double)min_len;
    if (l > (double)cap) l = (double)cap;
    len[i] = (int32_t)l;
    total += len[i];
  }
  free(raw);
  return total;
}

static int zipf_args_ok(int32_t m, int32_t n, int64_t target_nnz, double exponent,
                        int32_t min_len, int32_t max_len) {
  return m > 0 && n > 0 && target_nnz > 0 && exponent > 1.0 && min_len >= 1 &&
         max_len >= min_len && min_len <= n;
}

int64_t lpgen_planted_zipf_nnz(int32_t m, int32_t n, int64_t target_nnz, double exponent,
                               int32_t min_len, int32_t max_len, uint64_t seed) {
  if (!zipf_args_ok(m, n, target_nnz, exponent, min_len, max_len)) return -1;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  int32_t* len = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
  const int64_t total = zipf_lengths(g, m, n, target_nnz, exponent, min_len, max_len, len);
  free(len);
  free(g);
  return total;
}

int32_t lpgen_planted_zipf(int32_t m, int32_t n, int64_t target_nnz, double exponent,
                           int32_t min_len, int32_t max_len, uint64_t seed, lpgen_lp* lp) {
  if (!zipf_args_ok(m, n, target_nnz, exponent, min_len, max_len)) return 1;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  int32_t* len = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
  const int64_t nnz = zipf_lengths(g, m, n, target_nnz, exponent, min_len, max_len, len);
  if (nnz > INT32_MAX) {
    free(len);
    free(g);
    return 2;
  }
  /* Row-major draw: distinct uniform columns per row (rejection against a per-row stamp)
   * and the values, then a counting transpose into CSC. Rows are visited in ascending order,
   * so every column's row indices come out ascending. */
  int32_t* rcol = (int32_t*)malloc(sizeof(int32_t) * (size_t)nnz);
  double* rval = (double*)malloc(sizeof(double) * (size_t)nnz);
  int32_t* stamp = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  for (int32_t j = 0; j < n; ++j) stamp[j] = -1;
  const double ln10 = 2.30258509299404568402;
  int64_t at = 0;
  for (int32_t i = 0; i < m; ++i) {
    for (int32_t t = 0; t < len[i]; ++t) {
      int32_t c;
      do {
        c = unif_int(g, n);
      } while (stamp[c] == i);
      stamp[c] = i;
      rcol[at] = c;
      const double mag = det_exp(ln10 * unif_ab(g, -3.0, 3.0));
      rval[at] = unif(g) < 0.5 ? -mag : mag;
      ++at;
    }
  }
  lp->rows = m;
  lp->cols = n;
  lp->nnz = nnz;
  for (int32_t j = 0; j <= n; ++j) lp->col_starts[j] = 0;
  for (int64_t k = 0; k < nnz; ++k) lp->col_starts[rcol[k] + 1] += 1;
  for (int32_t j = 0; j < n; ++j) lp->col_starts[j + 1] += lp->col_starts[j];
  for (int32_t j = 0; j < n; ++j) stamp[j] = lp->col_starts[j];
  at = 0;
  for (int32_t i = 0; i < m; ++i) {
    for (int32_t t = 0; t < len[i]; ++t, ++at) {
      const int32_t slot = stamp[rcol[at]]++;
      lp->row_index[slot] = i;
      lp->values[slot] = rval[at];
    }
  }
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  for (int32_t j = 0; j < n; ++j) {
    box_point(g, &lp->x0[j], &z[j]);
    lp->col_lower[j] = 0.0;
    lp->col_upper[j] = 10.0;
  }
  for (int32_t i = 0; i < m; ++i) lp->lambda[i] = normal(g);
  finish_equalities(lp, z);
  free(z);
  free(stamp);
  free(rval);
  free(rcol);
  free(len);
  free(g);
  return 0;
}

int64_t lpgen_planted_nondegenerate_nnz(int32_t m, int32_t n, int32_t k) {
  (void)m;
  return (int64_t)n * k;
}

int32_t lpgen_planted_nondegenerate(int32_t m, int32_t n, int32_t k, uint64_t seed,
                                    lpgen_lp* lp) {
  if (m <= 0 || n < m || k <= 0 || k > m) return 1;
  mt64* g = (mt64*)malloc(sizeof(mt64));
  mt64_seed(g, seed);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  int32_t* basic_row = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  for (int32_t j = 0; j < n; ++j) perm[j] = j;
  for (int32_t j = n - 1; j > 0; --j) { /* Fisher-Yates */
    const int32_t r = unif_int(g, j + 1);
    const int32_t t = perm[j];
    perm[j] = perm[r];
    perm[r] = t;
  }
  for (int32_t j = 0; j < n; ++j) basic_row[j] = -1;
  for (int32_t p = 0; p < m; ++p) basic_row[perm[p]] = p;
  lp->rows = m;
  lp->cols = n;
  lp->nnz = (int64_t)n * k;
  int64_t at = 0;
  for (int32_t j = 0; j < n; ++j) {
    lp->col_starts[j] = (int32_t)at;
    int32_t* rows = lp->row_index + at;
    const int32_t p = basic_row[j];
    if (p >= 0) {
      /* Row p plus k - 1 distinct others, ascending. */
      int32_t t = 0;
      rows[t++] = p;
      while (t < k) {
        const int32_t r = unif_int(g, m);
        int dup = 0;
        for (int32_t s = 0; s < t; ++s) dup |= rows[s] == r;
        if (!dup) rows[t++] = r;
      }
      for (int32_t a = 1; a < k; ++a) { /* insertion sort */
        const int32_t v = rows[a];
        int32_t b = a;
        while (b > 0 && rows[b - 1] > v) {
          rows[b] = rows[b - 1];
          --b;
        }
        rows[b] = v;
      }
      for (int32_t s = 0; s < k; ++s) {
        const double v = normal(g);
        lp->values[at + s] = rows[s] == p ? (v < 0.0 ? -1.0 + v : 1.0 + v) : v;
      }
      lp->x0[j] = unif_ab(g, 0.1, 9.9);
      z[j] = 0.0;
    } else {
      pick_rows(g, 0, m, k, rows);
      for (int32_t s = 0; s < k; ++s) lp->values[at + s] = normal(g);
      if (unif(g) < 0.75) {
        lp->x0[j] = 0.0;
        z[j] = unif_ab(g, 0.1, 1.0);
      } else {
        lp->x0[j] = 10.0;
        z[j] = -unif_ab(g, 0.1, 1.0);
      }
    }
    at += k;
    lp->col_lower[j] = 0.0;
    lp->col_upper[j] = 10.0;
  }
  lp->col_starts[n] = (int32_t)at;
  for (int32_t i = 0; i < m; ++i) lp->lambda[i] = normal(g);
  finish_equalities(lp, z);
  free(perm);
  free(basic_row);
  free(z);
  free(g);
  return 0;
}

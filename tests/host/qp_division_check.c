/* qp_division_check.c -- the QP row pass's division against IEEE division, on the CPU.
 *
 * The row pass computes v / sigma as Markstein's correction of the product with the
 * correctly rounded reciprocal (qp_kernels.cu, divide(): q = RN(v inv), r = v - sigma q by
 * FMA, RN(q + r inv) unless r is 0 or NaN), with inv = RN(1 / sigma) computed on the host.
 * This program runs the same sequence with C's fma (correctly rounded in glibc) on random
 * pairs over 600 binades of v and 200 of sigma and on hand-picked cases, and counts the
 * quotients that differ from v / sigma in any bit. Built with -ffp-contract=off. Prints the
 * count and exits non-zero if it is not zero. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t state = 0x9E3779B97F4A7C15ull;

static uint64_t next(void) { /* splitmix64 */
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double uniform(void) { return (double)(next() >> 11) * 0x1.0p-53; }

static double divide(double v, double sigma, double inv) {
  const double q = v * inv;
  const double r = fma(-q, sigma, v);
  return (r == 0.0 || r != r) ? q : fma(r, inv, q);
}

static long long bad = 0, total = 0;

static void one(double v, double sigma) {
  const double inv = 1.0 / sigma;
  const double want = v / sigma;
  const double got = divide(v, sigma, inv);
  ++total;
  if (memcmp(&want, &got, sizeof(double)) != 0) {
    if (bad < 10) printf("differs: %a / %a = %a, sequence %a\n", v, sigma, want, got);
    ++bad;
  }
}

int main(int argc, char** argv) {
  long long count = argc > 1 ? atoll(argv[1]) : 20000000;
  const double picks[] = {0.0, -0.0, 1.0, -1.0, 3.0, 1.0 / 3.0, 0.1, 1e-300, 1e300, 7.0,
                          0x1.fffffffffffffp-1, 0x1.0000000000001p0, 123456789.0, -2.5};
  const int np = (int)(sizeof(picks) / sizeof(picks[0]));
  for (int a = 0; a < np; ++a) {
    for (int b = 0; b < np; ++b) {
      if (picks[b] > 0.0 && fabs(picks[a]) < 1e299 && picks[b] >= 1e-299) one(picks[a], picks[b]);
    }
  }
  for (long long k = 0; k < count; ++k) {
    /* sigma in [2^-100, 2^100), v of either sign in [2^-300, 2^300), and a share of v that are
     * multiples of sigma (exact quotients) or integers */
    const double sigma = ldexp(1.0 + uniform(), (int)(next() % 200) - 100);
    double v = ldexp(1.0 + uniform(), (int)(next() % 600) - 300);
    if (next() & 1) v = -v;
    switch (next() % 8) {
      case 0: v = sigma * (double)(int64_t)(next() % 1000000); break;
      case 1: v = (double)(int64_t)(next() % 2000001) - 1000000.0; break;
      default: break;
    }
    one(v, sigma);
  }
  printf("%lld of %lld quotients differ from IEEE division\n", bad, total);
  return bad == 0 ? 0 : 1;
}

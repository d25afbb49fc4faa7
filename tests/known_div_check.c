/* Checks the division by a divisor known in advance used by the convection
 * kernel (q0 = RN(x rb), r = x - b q0 by FMA, q = RN(q0 + r rb), rb = RN(1/b))
 * against IEEE division, bit for bit, on random dividends.
 * Usage: known_div_check <count> <seed> <b1> [b2 ...]; prints mismatches. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t rng_state;
static uint64_t next_u64(void) { /* splitmix64 */
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* A power-of-two divisor b = 2^p2: the exponent of a normal result is moved
 * on the bits, other results take x * 2^-p2 (exact reciprocal). */
#define NOT_POW2 (1 << 20)
static int pow2_exponent(double b) {
  int e = 0;
  return (frexp(b, &e) == 0.5 && e - 1 > -1000 && e - 1 < 1000) ? e - 1 : NOT_POW2;
}

static double div_known(double x, double b, double rb, int p2) {
  if (p2 != NOT_POW2) {
    uint64_t bits;
    memcpy(&bits, &x, 8);
    const int e = (int)((bits >> 52) & 0x7FF), ne = e - p2;
    if (e != 0 && e != 0x7FF && ne > 0 && ne < 0x7FF) {
      bits = (uint64_t)((int64_t)bits - (int64_t)p2 * ((int64_t)1 << 52));
      memcpy(&x, &bits, 8);
      return x;
    }
    return x * rb;
  }
  const double q0 = x * rb;
  const double r = fma(-q0, b, x);
  return (r == 0.0 || !isfinite(r)) ? q0 : fma(r, rb, q0);
}

static double random_dividend(void) {
  const uint64_t u = next_u64();
  switch (u & 3) {
    case 0: { /* any sign, exponent in [-60, 60], random mantissa */
      const int e = (int)((u >> 2) % 121) - 60;
      const double m = 1.0 + (double)(next_u64() >> 11) * 0x1.0p-53;
      return ldexp((u >> 10) & 1 ? -m : m, e);
    }
    case 1: /* velocities and their products in the benchmark's range */
      return ((double)(next_u64() >> 11) * 0x1.0p-53 - 0.5) * 10.0;
    case 2: /* small differences */
      return ((double)(next_u64() >> 11) * 0x1.0p-53 - 0.5) * 1e-6;
    default: { /* full random bit patterns of finite, normal numbers */
      double x;
      uint64_t bits = next_u64();
      memcpy(&x, &bits, 8);
      if (!isnormal(x) || fabs(x) > 1e300 || fabs(x) < 1e-290) x = 1.0;
      return x;
    }
  }
}

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  const long count = atol(argv[1]);
  rng_state = strtoull(argv[2], NULL, 10);
  long bad = 0;
  for (int a = 3; a < argc; ++a) {
    const double b = strtod(argv[a], NULL);
    const double rb = 1.0 / b;
    const int p2 = pow2_exponent(b);
    /* values at the ends of the range: zeros, subnormals, the largest
     * normals, infinities (results that leave the normal range) */
    const double edge[10] = {0.0, -0.0, 4.9e-324, -2.2e-310, 2.2250738585072014e-308, 1.7976931348623157e308,
                             -1e308, 1e300, INFINITY, -INFINITY};
    for (int q = 0; q < (p2 != NOT_POW2 ? 10 : 0); ++q) { /* the reciprocal-and-correction form is exact
                                                            only for normal x / b and x rb */
      const double got = div_known(edge[q], b, rb, p2), want = edge[q] / b;
      if (memcmp(&got, &want, 8) != 0) {
        if (bad < 10) printf("edge mismatch b=%.17g x=%.17g got %.17g want %.17g\n", b, edge[q], got, want);
        ++bad;
      }
    }
    for (long t = 0; t < count; ++t) {
      double x = random_dividend();
      if ((t & 15) == 0) x = (double)(long)(next_u64() % 2001 - 1000) * b; /* exact multiples */
      const double q = div_known(x, b, rb, p2), e = x / b;
      if (memcmp(&q, &e, 8) != 0) {
        if (bad < 10) printf("mismatch b=%.17g x=%.17g got %.17g want %.17g\n", b, x, q, e);
        ++bad;
      }
    }
  }
  const double zeros[2] = {0.0, -0.0};
  for (int z = 0; z < 2; ++z) {
    const double b = 0.0078125 * 0.41, q = div_known(zeros[z], b, 1.0 / b, NOT_POW2), e = zeros[z] / b;
    if (memcmp(&q, &e, 8) != 0) { printf("signed zero mismatch\n"); ++bad; }
  }
  printf("mismatches %ld\n", bad);
  return bad ? 1 : 0;
}

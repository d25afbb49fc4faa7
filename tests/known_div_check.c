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

static double div_known(double x, double b, double rb) {
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
    for (long t = 0; t < count; ++t) {
      double x = random_dividend();
      if ((t & 15) == 0) x = (double)(long)(next_u64() % 2001 - 1000) * b; /* exact multiples */
      const double q = div_known(x, b, rb), e = x / b;
      if (memcmp(&q, &e, 8) != 0) {
        if (bad < 10) printf("mismatch b=%.17g x=%.17g got %.17g want %.17g\n", b, x, q, e);
        ++bad;
      }
    }
  }
  const double zeros[2] = {0.0, -0.0};
  for (int z = 0; z < 2; ++z) {
    const double b = 0.0078125 * 0.41, q = div_known(zeros[z], b, 1.0 / b), e = zeros[z] / b;
    if (memcmp(&q, &e, 8) != 0) { printf("signed zero mismatch\n"); ++bad; }
  }
  printf("mismatches %ld\n", bad);
  return bad ? 1 : 0;
}
